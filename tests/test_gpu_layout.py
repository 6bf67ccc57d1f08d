"""The component layout: for Barnes-Hut fits whose affinity graph splits into
connected components of at most n / 4 points, the points are grouped by
component once, at the first periodic re-layout point (epoch 50), instead of
being re-laid out in Morton order every 50 epochs; every row's columns then
lie in its component's slot range. A layout is a permutation of the
optimisation state, so fits match the other layout up to summation order;
graphs with a large component keep the Morton layout."""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def separated(n, k, seed):
    """k clusters far apart in 16-D: the kNN graph's components are the clusters."""
    return blobs(n, 16, k, seed, spread=60.0)


def fit(gpu, X, idx, dist, y0, epochs, monkeypatch, layout, dtype=np.float32, seed=None):
    monkeypatch.setenv("BHTSNE_COMPONENT_LAYOUT", layout)
    t = gpu.TSNE(X.shape[0], D=2, dtype=dtype).perplexity(15.0).epochs(epochs)
    t = t.random_seed(seed) if seed is not None else t.initial_embedding(y0)
    t.barnes_hut_with_neighbors(0.5, (idx, dist.astype(dtype)))
    return t


@pytest.mark.parametrize("start", ["seeded", "caller"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_component_layout_matches_morton_layout(gpu, oracle, monkeypatch, dtype, start):
    """51 epochs in each layout from the same start: identical through epoch
    49, then one epoch in the component layout (composed with the Morton
    layout of a warm start's epoch 0) against one in the Morton layout."""
    X, lab = separated(20000, 8, 31)
    idx, dist = oracle.knn(X, 45)
    y0 = np.random.default_rng(32).normal(0, 1e-2, size=(20000, 2)).astype(dtype)
    seed = 33 if start == "seeded" else None
    tc = fit(gpu, X, idx, dist, y0, 51, monkeypatch, "2", dtype, seed)
    info = tc.layout_info()
    assert info["component_layout"] and info["largest_component"] == np.bincount(lab).max(), info
    assert tc.relayout_times()["count"] == (1 if start == "seeded" else 2)
    tm = fit(gpu, X, idx, dist, y0, 51, monkeypatch, "0", dtype, seed)
    assert not tm.layout_info()["component_layout"]
    ec, em = tc.embedding(), tm.embedding()
    assert np.all(np.isfinite(ec))
    tol = 1e-4 if dtype == np.float32 else 1e-9
    assert np.abs(ec - em).max() <= tol * np.abs(em).max(), np.abs(ec - em).max() / np.abs(em).max()


def test_component_layout_needs_small_components(gpu, oracle, monkeypatch):
    """Overlapping clusters: one component holds every point, so the fit keeps
    the Morton layout even when the component layout is forced."""
    X, _ = blobs(12000, 16, 8, 33, spread=1.0)
    idx, dist = oracle.knn(X, 45)
    y0 = np.random.default_rng(34).normal(0, 1e-4, size=(12000, 2)).astype(np.float32)
    t = fit(gpu, X, idx, dist, y0, 51, monkeypatch, "2")
    info = t.layout_info()
    assert not info["component_layout"] and info["largest_component"] > 12000 // 4, info


def test_component_layout_off_below_the_size_threshold(gpu, oracle, monkeypatch):
    """Unforced, fits below 65,536 points keep the Morton layout."""
    X, _ = separated(8000, 8, 35)
    idx, dist = oracle.knn(X, 45)
    y0 = np.random.default_rng(36).normal(0, 1e-4, size=(8000, 2)).astype(np.float32)
    monkeypatch.delenv("BHTSNE_COMPONENT_LAYOUT", raising=False)
    t = gpu.TSNE(8000, D=2).perplexity(15.0).epochs(51).initial_embedding(y0)
    t.barnes_hut_with_neighbors(0.5, (idx, dist))
    assert not t.layout_info()["component_layout"] and t.layout_info()["largest_component"] == 0


def test_component_layout_fit_matches_oracle(gpu, oracle, monkeypatch):
    """A whole fit in the component layout: final KL (both forms) within 1 %
    of the oracle's from the same kNN table and initial embedding."""
    X, _ = separated(6000, 8, 37)
    idx, dist = oracle.knn(X, 45)
    y0 = np.random.default_rng(38).normal(0, 1e-4, size=(6000, 2)).astype(np.float32)
    g = fit(gpu, X, idx, dist, y0, 500, monkeypatch, "2")
    assert g.layout_info()["component_layout"]
    o = oracle.TSNE(6000, 2).perplexity(15.0).epochs(500).initial_embedding(y0)
    o.barnes_hut_with_neighbors(0.5, idx.astype(np.uint64), dist)
    assert np.all(np.isfinite(g.embedding()))
    for quirk in (True, False):
        kg, ko = g.kl_divergence(quirk), o.kl_divergence(quirk)
        assert abs(kg - ko) / abs(ko) < 0.01, (quirk, kg, ko)
