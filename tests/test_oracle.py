"""Pins the CPU oracle against the reference crate's own known-answer tests
(tests/golden/reference_kats.json, each case citing the Rust test it comes
from). CPU only."""
import json
import os

import numpy as np
import pytest

from conftest import lcg_samples

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def lcg_cloud(n, dim, state):
    """src/tsne/arena.rs:482-492: (state >> 40) / 2^24 in f32."""
    out = np.empty(n * dim, np.float32)
    s = state
    for i in range(n * dim):
        s = (s * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
        out[i] = np.float32(np.float32(s >> 40) / np.float32(1 << 24))
    return out.reshape(n, dim)


def test_morton_known_z_order(oracle):
    for (a, b), code in KATS["morton2_known_z_order"]["cases"]:
        assert oracle.morton2(a, b) == code
    for (a, b, c), code in KATS["morton3_known_z_order"]["cases"]:
        assert oracle.morton3(a, b, c) == code
    codes = [oracle.morton2(*p) for p in KATS["morton2_sorting_groups_quadrants"]["ascending"]]
    assert codes == sorted(codes)


def test_morton_round_trip_bits(oracle):
    rng = np.random.default_rng(0x12345678)
    for _ in range(200):
        x, y = (int(v) for v in rng.integers(0, 2 ** 32, size=2))
        code = oracle.morton2(x, y)
        assert sum(((code >> (2 * i)) & 1) << i for i in range(32)) == x
        assert sum(((code >> (2 * i + 1)) & 1) << i for i in range(32)) == y


def test_quantize_kats(oracle):
    k = KATS["quantize_spans_bucket_range"]
    mn = np.array(k["min"], np.float32)
    inv = np.float32(k["scale"]) / np.array(k["extent"], np.float32)
    mb = k["max_bucket"]
    q = lambda p: [oracle.lib().orc_quantize_f32(float(p[a]), float(mn[a]), float(inv[a]), mb) for a in range(2)]
    assert q(k["low"]["point"]) == k["low"]["expect"]
    assert q(k["high"]["point"]) == k["high"]["expect"]
    mid = q(k["mid"]["point"])
    assert all(0 < v < mb for v in mid)
    z = KATS["quantize_zero_width_axis"]
    q0 = oracle.lib().orc_quantize_f32(z["point"][0], z["min"][0], z["inv_scale"][0], mb)
    q1 = oracle.lib().orc_quantize_f32(z["point"][1], z["min"][1], np.float32(z["inv_scale"][1]), mb)
    assert q0 == z["expect_axis0"] and q1 > 0


def test_search_beta_known_answer(oracle):
    k = KATS["search_beta_below_one"]
    d = np.array(k["distances"], np.float64)[None, :]
    p, _ = oracle.search_beta(d, k["perplexity"])
    p = p[0][p[0] > 0]
    eff = np.exp(-(p * np.log(p)).sum())
    assert abs(eff - k["perplexity"]) < k["effective_perplexity_tolerance"]


def test_fft_round_trip_and_convolution(oracle):
    k = KATS["fft_round_trip_2d"]
    m = k["m"]
    rng = np.random.default_rng(0xABCD)
    x = rng.uniform(-0.5, 0.5, (m, m))
    re, im = oracle.fft(x, np.zeros_like(x))
    re, im = oracle.fft(re, im, inverse=True)
    assert np.max(np.abs(re / (m * m) - x)) < k["tolerance"]
    k1 = KATS["fft_round_trip_1d"]
    x1 = rng.uniform(-0.5, 0.5, k1["m"])
    r1, i1 = oracle.fft(x1, np.zeros_like(x1))
    r1, i1 = oracle.fft(r1, i1, inverse=True)
    assert np.max(np.abs(r1 / k1["m"] - x1)) < k1["tolerance"]
    kc = KATS["fft_circular_convolution_2d"]
    m = kc["m"]
    a = rng.uniform(-0.5, 0.5, (m, m))
    b = rng.uniform(-0.5, 0.5, (m, m))
    direct = np.zeros((m, m))
    for i in range(m):
        for j in range(m):
            direct[i, j] = sum(a[(i - u) % m, (j - v) % m] * b[u, v] for u in range(m) for v in range(m))
    ar, ai = oracle.fft(a, np.zeros_like(a))
    br, bi = oracle.fft(b, np.zeros_like(b))
    pr, pi = ar * br - ai * bi, ar * bi + ai * br
    cr, _ = oracle.fft(pr, pi, inverse=True)
    assert np.max(np.abs(cr / (m * m) - direct)) < kc["tolerance"]


def test_fft_smooth_lengths(oracle):
    # 7-smooth lengths used by the interpolation grid (src/tsne/interpolation.rs:364-378)
    assert [oracle.next_smooth(n) for n in (1, 11, 13, 59, 97, 121)] == [1, 12, 14, 60, 98, 125]
    for m in (60, 98, 30):
        x = np.random.default_rng(m).uniform(-1, 1, m)
        r, i = oracle.fft(x, np.zeros_like(x))
        ref = np.fft.fft(x)
        assert np.max(np.abs(r - ref.real)) < 1e-9 and np.max(np.abs(i - ref.imag)) < 1e-9


def test_lagrange_partition_and_cardinality(oracle):
    k = KATS["lagrange_partition_of_unity"]
    for s in range(k["steps"]):
        assert abs(oracle.lagrange_weights(s / 10.0).sum() - 1.0) < k["tolerance"]
    for j in range(3):
        w = oracle.lagrange_weights((j + 0.5) / 3.0)
        assert np.allclose(w, np.eye(3)[j], atol=k["tolerance"])


def brute_repulsion(y):
    diff = y[:, None, :] - y[None, :, :]
    d2 = (diff ** 2).sum(-1)
    c = 1.0 / (1.0 + d2)
    np.fill_diagonal(c, 0.0)
    return ((c ** 2)[:, :, None] * diff).sum(1), c.sum()


@pytest.mark.parametrize("case,D", [("interpolation_vs_brute_force_2d", 2), ("interpolation_vs_brute_force_1d", 1)])
def test_interpolation_vs_brute_force(oracle, case, D):
    k = KATS[case]
    rng = np.random.default_rng(0xBADC0DE)
    y = rng.uniform(k["uniform"][0], k["uniform"][1], (k["n"], D))
    neg, z, _ = oracle.fit_repulsion(y)
    fr, zr = brute_repulsion(y)
    assert abs(z - zr) / zr < k["z_rel"]
    assert np.linalg.norm(neg - fr) / np.linalg.norm(fr) < k["force_rel_l2"]


def test_arena_conservation_and_root(oracle):
    k = KATS["arena_conserves_points_2d"]
    y = lcg_samples(k["n"], 2, k["lcg_seed"]) + np.float32(k["offset"])
    t = oracle.bh_tree(y)
    leaves = t["first_child"] == 0xFFFFFFFF
    assert t["count"][0] == k["n"] and t["count"][leaves].sum() == k["n"]
    k3 = KATS["arena_conserves_points_3d"]
    t3 = oracle.bh_tree(lcg_samples(k3["n"], 3, k3["lcg_seed"]))
    assert t3["count"][0] == k3["n"]
    kr = KATS["arena_root_com_is_mean"]
    y = lcg_cloud(kr["n"], 2, kr["lcg_seed"])
    t = oracle.bh_tree(y)
    assert np.all(np.abs(t["com"][0] - y.mean(0)) < kr["tolerance"])


def quantize_np(y, bits):
    """Quantisation of src/tsne/morton.rs:103-120 in float32 numpy arithmetic."""
    mn, mx = y.min(0), y.max(0)
    ext = (mx - mn).astype(np.float32)
    inv = np.where(ext > 0, np.float32(2.0 ** bits) / np.where(ext > 0, ext, 1), 0).astype(np.float32)
    scaled = np.floor(((y - mn).astype(np.float32) * inv).astype(np.float32))
    q = np.where(scaled > 0, np.minimum(scaled.astype(np.float64), 2.0 ** bits - 1), 0).astype(np.uint64)
    return q, mn, ext


def test_arena_coms_within_cells(oracle):
    """check_coms_within_cells (src/tsne/arena.rs:432-463) on the oracle's arena."""
    k = KATS["arena_coms_within_cells"]
    y = lcg_samples(k["n"], 2, k["lcg_seed"]) + np.float32(k["offset"])
    t = oracle.bh_tree(y)
    bits = 32
    q, mn, ext = quantize_np(y, bits)
    codes = [oracle.morton2(int(a), int(b)) for a, b in q]
    perm = sorted(range(len(y)), key=lambda i: (codes[i], i))
    for v in range(len(t["count"])):
        lvl = int(t["level"][v])
        rep = perm[int(t["range_start"][v])]
        for a in range(2):
            width = np.float32(ext[a] / np.float32(2.0 ** lvl))
            cell = np.float32(int(q[rep, a]) >> (bits - lvl))
            low = np.float32(mn[a] + cell * width)
            high = np.float32(low + width)
            slack = np.float32(k["slack_fraction"]) * (ext[a] + max(abs(low), abs(high)))
            assert low - slack <= t["com"][v, a] <= high + slack


def test_arena_degenerate_inputs(oracle):
    k = KATS["arena_duplicates_collapse"]
    y = np.full((k["n"], 2), k["value"], np.float32)
    t = oracle.bh_tree(y)
    assert len(t["count"]) == k["expect_nodes"] and t["count"][0] == k["n"]
    assert t["first_child"][0] == 0xFFFFFFFF
    p = np.array([KATS["arena_single_point"]["point"]], np.float32)
    t = oracle.bh_tree(p)
    assert len(t["count"]) == 1 and np.array_equal(t["com"][0], p[0])
    assert oracle.bh_tree(np.zeros((0, 2), np.float32))["count"].size == 0


def test_learning_rate_formula(oracle):
    k = KATS["learning_rate"]
    for n, ex, want in k["cases"]:
        t = oracle.TSNE(n).early_exaggeration(ex)
        assert t.get("learning_rate") == pytest.approx(want, rel=1e-6)
    lo, hi = k["n10000_range"]
    assert lo <= oracle.TSNE(10000).get("learning_rate") <= hi
    n, ex = k["halving_exaggeration_doubles"]
    a = oracle.TSNE(n).get("learning_rate")
    b = oracle.TSNE(n).early_exaggeration(ex).get("learning_rate")
    assert b == pytest.approx(2 * a, rel=1e-6)


def cluster_data(k):
    state = k["lcg_seed"]
    vals = []
    for c in k["centres"]:
        for _ in range(k["n_per_cluster"] * k["dim"]):
            state = (state * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
            r = np.float32(np.float32(state >> 33) / np.float32(4294967295.0)) - np.float32(0.5)
            vals.append(np.float32(c) + np.float32(k["noise_scale"]) * r)
    return np.array(vals, np.float32).reshape(-1, k["dim"])


def same_cluster_fraction(emb, n_per):
    e = emb.reshape(-1, 2).astype(np.float64)
    d = ((e[:, None, :] - e[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    nn = d.argmin(1)
    lab = np.arange(len(e)) < n_per
    return float(np.mean(lab == lab[nn]))


def test_clusters_separate(oracle):
    k = KATS["clusters_separate_large_scale"]
    X = cluster_data(k)
    t = oracle.TSNE(len(X)).perplexity(k["perplexity"]).epochs(k["epochs"])
    t.barnes_hut(k["theta"], X)
    assert same_cluster_fraction(t.embedding(), k["n_per_cluster"]) > k["min_fraction"]


def test_no_collapse(oracle):
    k = KATS["no_collapse"]
    X = lcg_samples(k["n"], k["dim"], k["lcg_seed"])
    t = oracle.TSNE(k["n"]).perplexity(k["perplexity"]).epochs(k["epochs"])
    t.barnes_hut(k["theta"], X)
    e = t.embedding().reshape(-1, 2)
    distinct = {(int(round(a * 100)), int(round(b * 100))) for a, b in e}
    assert len(distinct) > k["min_distinct_fraction"] * k["n"]


def test_kl_finite_nonnegative(oracle):
    k = KATS["kl_finite_nonnegative"]
    X = lcg_samples(k["n"], k["dim"], k["lcg_seed"])
    t = oracle.TSNE(k["n"]).perplexity(k["perplexity"]).epochs(k["epochs"])
    assert t.kl_divergence() is None
    t.barnes_hut(0.5, X)
    kl = t.kl_divergence()
    assert np.isfinite(kl) and kl >= 0
    d = ((X[:, None, :].astype(np.float32) - X[None, :, :]) ** 2).sum(-1).astype(np.float32)
    te = oracle.TSNE(k["n"]).perplexity(k["perplexity"]).epochs(k["epochs"])
    te.exact(d)
    kl = te.kl_divergence()
    assert np.isfinite(kl) and kl >= 0


def test_with_neighbors_equals_metric_path(oracle):
    k = KATS["with_neighbors_equals_metric_path"]
    X = lcg_samples(k["n"], k["dim"], k["lcg_seed"])
    seed = lcg_samples(k["n"], 2, k["seed_lcg"])
    kk = int(3 * k["perplexity"])
    idx, dist = oracle.knn(X, kk)
    a = oracle.TSNE(k["n"]).perplexity(k["perplexity"]).epochs(k["epochs"]).initial_embedding(seed)
    a.barnes_hut(k["theta"], X)
    b = oracle.TSNE(k["n"]).perplexity(k["perplexity"]).epochs(k["epochs"]).initial_embedding(seed)
    b.barnes_hut_with_neighbors(k["theta"], idx.astype(np.uint64), dist)
    assert np.array_equal(a.embedding(), b.embedding())


def test_symmetrize_properties(oracle):
    X = lcg_samples(300, 5, 3)
    idx, dist = oracle.knn(X, 30)
    p, _ = oracle.search_beta(dist, 10.0)
    rows, cols, vals = oracle.symmetrize(idx, p)
    n = len(X)
    dense = np.zeros((n, n))
    for i in range(n):
        for e in range(rows[i], rows[i + 1]):
            dense[i, cols[e]] += vals[e]
    assert np.allclose(dense, dense.T)
    assert abs(vals.sum() - n) / n < 1e-5  # each conditional row sums to ~1, halved twice over
    norm = oracle.normalize(vals, 1.0)
    assert abs(norm.sum() - 1.0) < 0.05


@pytest.mark.parametrize("D,bits", [(4, 16), (5, 25), (6, 21), (7, 18)])
def test_morton_wide_codecs(oracle, D, bits):
    """src/tsne/morton/d4.rs-d7.rs: bit b of axis a at code bit b * D + a
    (d5.rs-d7.rs spread through nibble tables into a u128; d4.rs by masks)."""
    rng = np.random.default_rng(40 + D)
    for _ in range(100):
        c = [int(v) for v in rng.integers(0, 2 ** bits, size=D)]
        code = oracle.morton(c)
        assert code < (1 << (D * bits))
        for a in range(D):
            assert sum(((code >> (b * D + a)) & 1) << b for b in range(bits)) == c[a]
    # the top bit of the last axis is the code's most significant bit
    top = [0] * D
    top[-1] = 1 << (bits - 1)
    assert oracle.morton(top) == 1 << (D * bits - 1)


@pytest.mark.parametrize("D", [4, 5, 6, 7])
def test_oracle_wide_arena_matches_exact_repulsion(oracle, D):
    """The D = 4..7 arena conserves points and, with a tiny theta, its
    repulsion equals the exact sum over all other points."""
    rng = np.random.default_rng(70 + D)
    y = rng.normal(0, 2.0, size=(600, D)).astype(np.float64)
    t = oracle.bh_tree(y)
    leaves = t["first_child"] == 0xFFFFFFFF
    assert t["count"][0] == 600 and t["count"][leaves].sum() == 600
    neg, q, z = oracle.bh_repulsion(y, 1e-6)
    d = y[:, None, :] - y[None, :, :]
    w = 1.0 / (1.0 + (d ** 2).sum(-1))
    np.fill_diagonal(w, 0.0)
    ref_neg = ((w ** 2)[:, :, None] * d).sum(1)
    assert abs(z - w.sum()) / w.sum() < 1e-12
    assert np.max(np.abs(neg - ref_neg)) < 1e-12 * max(1.0, np.abs(ref_neg).max())
