"""T = f64 (the reference's `tSNE::<f64, ..>`, as in examples/mnist_pca_tsne.rs):
every stage and a full fit against the oracle run in f64."""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def data64(n, dim, seed):
    X, lab = blobs(n, dim, 6, seed)
    return X.astype(np.float64), lab


def test_knn_f64_exact(gpu, oracle):
    X, _ = data64(2500, 40, 3)
    gi, gd = gpu.knn_euclidean(X, 60)
    oi, od = oracle.knn(X, 60)
    assert gd.dtype == np.float64
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


def test_affinities_f64(gpu, oracle):
    X, _ = data64(1500, 20, 4)
    oi, od = oracle.knn(X, 60)
    gp, _ = gpu.conditional_p(od, 20.0)
    op, _ = oracle.search_beta(od, 20.0)
    assert np.max(np.abs(gp - op) / np.maximum(op, 1e-300)) < 1e-5
    grows, gcols, gvals = gpu.symmetrize(oi, op)
    orows, ocols, ovals = oracle.symmetrize(oi, op)
    assert np.array_equal(grows, orows) and np.array_equal(gcols, ocols) and np.array_equal(gvals, ovals)


@pytest.mark.parametrize("D", [2, 3, 5])
def test_bh_gradient_f64(gpu, oracle, D):
    X, _ = data64(2000, 20, 5)
    oi, od = oracle.knn(X, 60)
    op, _ = oracle.search_beta(od, 20.0)
    rows, cols, vals = oracle.symmetrize(oi, op)
    vals = oracle.normalize(vals, 12.0)
    y = np.random.default_rng(D).normal(0, 3.0, size=(2000, D))
    pos, neg, z = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
    opos = oracle.edge_forces(y, rows, cols, vals)
    oneg, _, oz = oracle.bh_repulsion(y, 0.5)
    assert rel_l2(pos, opos) < 1e-12
    assert rel_l2(neg, oneg) < 1e-9
    assert abs(z - oz) / oz < 1e-9


def test_fit_sne_gradient_f64(gpu, oracle):
    y = np.random.default_rng(11).uniform(-15, 15, size=(3000, 2))
    rows = np.zeros(3001, np.uint64)
    _, neg, z = gpu.gradient(gpu.METHOD_FIT_SNE, y, rows, np.zeros(0, np.uint32), np.zeros(0, np.float64))
    oneg, oz, _ = oracle.fit_repulsion(y)
    assert rel_l2(neg, oneg) < 1e-9
    assert abs(z - oz) / abs(oz) < 1e-9


@pytest.mark.parametrize("method", ["bh", "fit"])
def test_fit_f64_final_kl_matches_oracle(gpu, oracle, method):
    X, _ = data64(1500, 30, 6)
    idx, dist = oracle.knn(X, 60)
    seed = np.random.default_rng(2).normal(0, 1e-4, size=(1500, 2))
    g = gpu.TSNE(1500, dtype=np.float64).perplexity(20).epochs(500).initial_embedding(seed)
    o = oracle.TSNE(1500, dtype=np.float64).perplexity(20).epochs(500).initial_embedding(seed)
    if method == "bh":
        g.barnes_hut_with_neighbors(0.5, (idx, dist))
        o.barnes_hut_with_neighbors(0.5, idx.astype(np.uint64), dist)
    else:
        g.fit_sne_with_neighbors((idx, dist))
        o.fit_sne_with_neighbors(idx.astype(np.uint64), dist)
    assert g.embedding().dtype == np.float64
    for quirk in (True, False):
        kg, ko = g.kl_divergence(quirk), o.kl_divergence(quirk)
        assert abs(kg - ko) / abs(ko) < 0.01, (method, quirk, kg, ko)
