"""Degenerate inputs and cache edge cases, against the oracle where a value
is defined and against the reference's tests (src/test.rs) for the builder
semantics."""
import numpy as np
import pytest

from conftest import blobs, lcg_samples

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def affinities_of(oracle, X, k, perp):
    oi, od = oracle.knn(X, k)
    op, _ = oracle.search_beta(od, perp)
    rows, cols, vals = oracle.symmetrize(oi, op)
    return rows, cols, oracle.normalize(vals, 12.0)


@pytest.mark.parametrize("D", [2, 3])
def test_bh_gradient_with_coincident_points(gpu, oracle, D):
    """Exact duplicates share a leaf; a query's own leaf (distance 0) is
    skipped with its duplicates, as the arena traversal does
    (src/tsne/arena.rs:360-362)."""
    X, _ = blobs(600, 8, 3, 9)
    rows, cols, vals = affinities_of(oracle, X, 30, 10.0)
    rng = np.random.default_rng(1)
    y = rng.normal(0, 2.0, size=(600, D)).astype(np.float32)
    y[100:160] = y[99]          # a block of 61 identical points
    y[300:302] = y[299]
    pos, neg, z = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
    opos = oracle.edge_forces(y, rows, cols, vals)
    oneg, _, oz = oracle.bh_repulsion(y, 0.5)
    assert rel_l2(pos, opos) < 1e-5
    assert rel_l2(neg, oneg) < 1e-4
    assert abs(z - oz) / oz < 1e-4


def test_gradient_of_a_collapsed_embedding(gpu, oracle):
    """All points at one location. Barnes-Hut: zero extent gives inv_scale 0
    and a single leaf, which every query skips (src/tsne/arena.rs:156-163,
    368-372), so the repulsion and Z are exactly zero. FIt-SNE: the extent is
    floored at min_positive (src/tsne/interpolation.rs:116), the box width is
    then subnormal and its reciprocal (line 163) overflows to infinity, so the
    offset (y - min) * inv_box_width is 0 * inf = NaN and the reference's
    forces and Z are NaN; the GPU path reproduces that."""
    X, _ = blobs(400, 8, 2, 10)
    rows, cols, vals = affinities_of(oracle, X, 30, 10.0)
    for dt in (np.float32, np.float64):
        y = np.full((400, 2), 0.25, dt)
        r, c, v = rows, cols, vals.astype(dt)
        pos, neg, z = gpu.gradient(gpu.METHOD_BARNES_HUT, y, r, c, v, theta=0.5)
        oneg, _, oz = oracle.bh_repulsion(y, 0.5)
        assert np.all(pos == 0) and np.all(neg == 0) and z == 0
        assert np.all(oneg == 0) and oz == 0
        _, neg, z = gpu.gradient(gpu.METHOD_FIT_SNE, y, r, c, v)
        oneg, oz, _ = oracle.fit_repulsion(y)
        assert np.all(np.isnan(oneg)) and np.isnan(oz)
        assert np.all(np.isnan(neg)) and np.isnan(z)
        # any positive extent is finite on both sides
        y[0, 0] += dt(1e-3)
        _, neg, z = gpu.gradient(gpu.METHOD_FIT_SNE, y, r, c, v)
        oneg, oz, _ = oracle.fit_repulsion(y)
        assert np.all(np.isfinite(neg)) and np.isfinite(z)
        assert abs(z - oz) <= 1e-4 * abs(oz)
        assert np.abs(neg - oneg).max() <= 1e-3 * np.abs(oneg).max() + 1e-3


@pytest.mark.parametrize("method", ["bh", "fit", "exact"])
def test_smallest_dataset_for_the_perplexity(gpu, method):
    """check_perplexity (src/tsne/mod.rs:55-59): n - 1 >= 3 floor(perplexity)."""
    perp = 5.0
    X = lcg_samples(16, 4, 3)
    t = gpu.TSNE(X).perplexity(perp).epochs(60)
    getattr(t, {"bh": "barnes_hut", "fit": "fit_sne", "exact": "exact"}[method])(
        *([0.5] if method == "bh" else []))
    assert np.all(np.isfinite(t.embedding()))
    small = gpu.TSNE(X[:15]).perplexity(perp).epochs(10)
    with pytest.raises(gpu.BhtsneError, match="perplexity is too large"):
        getattr(small, {"bh": "barnes_hut", "fit": "fit_sne", "exact": "exact"}[method])(
            *([0.5] if method == "bh" else []))


def test_fit_with_many_duplicate_inputs(gpu):
    """Duplicate input rows have zero distances to each other; the fit stays
    finite and duplicates land together."""
    base, _ = blobs(200, 6, 3, 12)
    X = np.concatenate([base, base, base[:50]])
    for method in ("bh", "fit"):
        t = gpu.TSNE(X).perplexity(10).epochs(300)
        t.barnes_hut(0.5) if method == "bh" else t.fit_sne()
        e = t.embedding().reshape(-1, 2)
        assert np.all(np.isfinite(e))
        assert np.median(np.linalg.norm(e[:200] - e[200:400], axis=1)) < 0.1 * np.ptp(e)


def test_cached_affinities_random_seed(gpu):
    """src/test.rs:1480-1514: injected affinities with no initial embedding
    start from the random draw."""
    X = lcg_samples(50, 4, 7)
    ref = gpu.TSNE(X).perplexity(10).epochs(200)
    ref.barnes_hut(0.5)
    t = gpu.TSNE(X).perplexity(10).epochs(50).with_affinities(ref.affinities())
    t.barnes_hut(0.5)
    e = t.embedding()
    assert e.size == 100 and np.all(np.isfinite(e)) and np.any(e != 0)


def test_cached_affinities_discarded_on_dataset_mismatch(gpu):
    """src/test.rs:1516-1553: affinities of another dataset size are dropped
    and rebuilt, not used."""
    small = lcg_samples(50, 4, 7)
    t = gpu.TSNE(small).perplexity(10).epochs(200)
    t.barnes_hut(0.5)
    aff = t.affinities()
    large = lcg_samples(100, 4, 7)
    u = gpu.TSNE(large).perplexity(10).with_affinities(aff)
    u.barnes_hut(0.5)
    e = u.embedding()
    assert e.size == 200 and np.all(np.isfinite(e))
    assert u.affinities().rows.size == 101
    fresh = gpu.TSNE(large).perplexity(10)
    fresh.barnes_hut(0.5)
    assert np.array_equal(u.affinities().values, fresh.affinities().values)


def test_cached_affinities_reset_stop_lying_flag(gpu, oracle):
    """src/test.rs:1624-1688: a second fit on the same instance takes the
    cached-affinities path and exaggerates P again until the stop-lying epoch,
    so it equals a fresh fit from the same seed."""
    X = lcg_samples(80, 4, 42)
    idx, dist = oracle.knn(X, 30)
    pre = gpu.TSNE(X).perplexity(10).epochs(20)
    pre.barnes_hut(0.5)
    seed = pre.embedding()
    b = gpu.TSNE(X).perplexity(10).stop_lying_epoch(5).epochs(20)
    b.barnes_hut_with_neighbors(0.5, (idx, dist))
    b.epochs(20).initial_embedding(seed)
    b.barnes_hut_with_neighbors(0.5, (idx, dist))
    c = gpu.TSNE(X).perplexity(10).stop_lying_epoch(5).epochs(20).initial_embedding(seed)
    c.barnes_hut_with_neighbors(0.5, (idx, dist))
    assert np.array_equal(b.embedding(), c.embedding())
    # without the reset the exaggeration would stay on for all 20 epochs
    d = gpu.TSNE(X).perplexity(10).stop_lying_epoch(20).epochs(20).initial_embedding(seed)
    d.barnes_hut_with_neighbors(0.5, (idx, dist))
    assert not np.array_equal(b.embedding(), d.embedding())


def test_with_affinities_adopts_perplexity(gpu):
    """src/test.rs:1690-1707."""
    X = np.arange(800, dtype=np.float32).reshape(200, 4)
    t = gpu.TSNE(X).perplexity(30).epochs(20)
    t.barnes_hut(0.5)
    u = gpu.TSNE(X).perplexity(5).with_affinities(t.affinities())
    assert u.affinities().perplexity == pytest.approx(30.0)
