"""The attractive pass over the 2-D blocked copy of P (compute_edge_forces,
src/tsne/arena.rs:398-427): points in blocks of 2^k slots, each column tile of
y staged in shared memory by bulk copies while its entries are summed. It is
used for large fits in D <= 3; BHTSNE_ATTR_BLOCKED=0 selects the row-task pass
instead. Both against the oracle, and against each other inside fits (the
blocked copy is read through the slot maps of the locality layout, rebuilt at
each re-layout, and rescaled when the exaggeration stops)."""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def knn_graph(gpu, oracle, n, dim, k, seed, dtype):
    X, lab = blobs(n, dim, 12, seed)
    gi, gd = gpu.knn_euclidean(X, k)
    op, _ = oracle.search_beta(gd, k / 3.0)
    rows, cols, vals = oracle.symmetrize(gi, op)
    return X, rows, cols, oracle.normalize(vals, 12.0).astype(dtype)


@pytest.mark.parametrize("dtype,D,n", [(np.float32, 2, 70000), (np.float32, 3, 40000), (np.float32, 1, 140000),
                                       (np.float64, 2, 40000)])
def test_blocked_pass_matches_oracle_and_task_pass(gpu, oracle, monkeypatch, dtype, D, n):
    """At least eight row blocks (2^13 points for f32 in 2-D, 2^12 in 3-D and
    for f64, 2^14 in 1-D), so the blocked pass is the one that runs; the last
    block and tile are partial. Within 1e-5 (f32; 1e-12 f64) of the oracle and
    1e-6 of the task pass."""
    _, rows, cols, vals = knn_graph(gpu, oracle, n, 16, 45, 41 + D, dtype)
    y = np.random.default_rng(42).normal(0, 8.0, size=(n, D)).astype(dtype)
    method = gpu.METHOD_FIT_SNE if D <= 2 else gpu.METHOD_BARNES_HUT
    monkeypatch.setenv("BHTSNE_ATTR_BLOCKED", "1")
    pos_b, _, _ = gpu.gradient(method, y, rows, cols, vals)
    monkeypatch.setenv("BHTSNE_ATTR_BLOCKED", "0")
    pos_t, _, _ = gpu.gradient(method, y, rows, cols, vals)
    opos = oracle.edge_forces(y, rows, cols, vals)
    bar = 1e-5 if dtype == np.float32 else 1e-12
    assert rel_l2(pos_b, opos) < bar
    assert rel_l2(pos_t, opos) < bar
    assert rel_l2(pos_b, pos_t) < (1e-6 if dtype == np.float32 else 1e-13)


def test_blocked_pass_is_deterministic(gpu, oracle, monkeypatch):
    """Rows are summed by one warp per tile and tiles in order: the same
    forces bit for bit on every call."""
    _, rows, cols, vals = knn_graph(gpu, oracle, 80000, 16, 60, 43, np.float32)
    y = np.random.default_rng(44).normal(0, 8.0, size=(80000, 2)).astype(np.float32)
    monkeypatch.setenv("BHTSNE_ATTR_BLOCKED", "1")
    a, _, _ = gpu.gradient(gpu.METHOD_FIT_SNE, y, rows, cols, vals)
    b, _, _ = gpu.gradient(gpu.METHOD_FIT_SNE, y, rows, cols, vals)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("method", ["bh", "fit"])
def test_blocked_pass_inside_fits(gpu, monkeypatch, method):
    """A warm-started 70k-point fit with the exaggeration stopped at epoch 2
    (the blocked copy's values rescaled) against the task pass re-laid out
    every two epochs: after 5 epochs the embeddings agree up to summation
    order. The blocked pass needs no locality, so its fit is not re-laid out."""
    X, _ = blobs(70000, 16, 12, 45)
    y0 = np.random.default_rng(46).normal(0, 1.0, size=(70000, 2)).astype(np.float32)
    out = {}
    monkeypatch.setenv("BHTSNE_RENUMBER_EVERY", "2")
    for blocked in ("1", "0"):
        monkeypatch.setenv("BHTSNE_ATTR_BLOCKED", blocked)
        t = gpu.TSNE(X).perplexity(15).epochs(5).stop_lying_epoch(2).momentum_switch_epoch(2).initial_embedding(y0)
        t.barnes_hut(0.5) if method == "bh" else t.fit_sne()
        out[blocked] = t.embedding()
        assert t.relayout_times()["count"] == (0 if blocked == "1" else 3)
    e1, e0 = out["1"], out["0"]
    assert np.all(np.isfinite(e1))
    assert np.abs(e1 - e0).max() <= 1e-4 * np.abs(e0).max(), np.abs(e1 - e0).max() / np.abs(e0).max()
