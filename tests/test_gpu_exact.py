"""The exact method and the fused update against the oracle.

The exact path (src/lib.rs:489-646) has its own quirks that the sparse paths
do not exercise: P keeps the diagonal (search_beta over full rows, the zero
self-distance included), the symmetrisation is p + p^T without halving, Q
includes q_ii = 1 so Z counts n, and the gradient carries no factor 4. The
update tests pin gradient_descent_step + zero_mean (src/tsne/mod.rs:470-516,
:534-568) at fixed inputs, including +0 and -0 gradients and velocities where
Rust's `signum` decides the gain.
"""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu

TOL = {np.float32: 1e-4, np.float64: 1e-9}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def sq_dist_matrix(X):
    """Squared Euclidean distances in X's type, summed over the dimensions in
    order (the arithmetic of the reference's README closure)."""
    n, dim = X.shape
    s = np.zeros((n, n), X.dtype)
    for c in range(dim):
        d = X[:, None, c] - X[None, :, c]
        s = s + d * d
    return s


def exact_p(oracle, X, perplexity, exaggeration=12.0):
    p = oracle.exact_affinities(sq_dist_matrix(X), perplexity)
    return oracle.normalize(p.ravel(), exaggeration).reshape(p.shape)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("D", [1, 2, 3])
def test_exact_gradient_at_fixed_y(gpu, oracle, dtype, D):
    """bhtsne_gradient(EXACT) against the oracle's exact gradient at the same
    y and dense P (exaggerated, diagonal included): dy within 1e-4 relative
    L2 in f32 (1e-9 in f64), Z (which counts the n diagonal entries) alike."""
    X, _ = blobs(700, 12, 4, 11)
    X = X.astype(dtype)
    p = exact_p(oracle, X, 30.0)
    assert np.all(np.diag(p) > 0), "the exact P keeps its diagonal"
    rng = np.random.default_rng(100 + D)
    y = rng.normal(0.0, 2.0, size=(700, D)).astype(dtype)
    dy, _, z = gpu.gradient(gpu.METHOD_EXACT, y, None, None, p)
    ody, oz = oracle.exact_gradient(p, y)
    assert oz > 700
    assert rel_l2(dy, ody) < TOL[dtype]
    assert abs(z - oz) / oz < TOL[dtype]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_exact_gradient_after_stop_lying(gpu, oracle, dtype):
    """The same at an un-exaggerated P and a spread-out embedding, where the
    repulsive term dominates and the attractive and repulsive sums cancel."""
    X, _ = blobs(500, 8, 6, 12)
    X = X.astype(dtype)
    p = exact_p(oracle, X, 20.0, exaggeration=1.0)
    rng = np.random.default_rng(12)
    y = rng.normal(0.0, 15.0, size=(500, 2)).astype(dtype)
    dy, _, z = gpu.gradient(gpu.METHOD_EXACT, y, None, None, p)
    ody, oz = oracle.exact_gradient(p, y)
    assert rel_l2(dy, ody) < TOL[dtype]
    assert abs(z - oz) / oz < TOL[dtype]


def _exact_pair(gpu, oracle, X, variant, dtype, epochs, perplexity, y0):
    g = gpu.TSNE(X, dtype=dtype).perplexity(perplexity).epochs(epochs).initial_embedding(y0)
    o = oracle.TSNE(len(X), 2, dtype).perplexity(perplexity).epochs(epochs).initial_embedding(y0)
    sq = sq_dist_matrix(X)
    if variant == "sqeuclidean":
        g.exact("sqeuclidean")
        o.exact(sq)
    elif variant == "euclidean":
        g.exact("euclidean")
        o.exact(np.sqrt(sq))
    else:
        # an arbitrary metric given as its matrix: L1 distances; the lower
        # triangle is garbage and must not be read
        m = np.abs(X[:, None, :] - X[None, :, :]).sum(-1).astype(dtype)
        m[np.tril_indices(len(X), -1)] = -7.0
        g.exact(m)
        o.exact(m)
    return g, o


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("variant", ["sqeuclidean", "euclidean", "matrix"])
def test_exact_fit_first_epochs(gpu, oracle, variant, dtype):
    """The exact fit's first epochs from the same initial embedding: the
    displacement y - y0 after 3 epochs depends on P of each variant (the
    squared distance that search_beta squares again, the Euclidean distance,
    and a caller-supplied matrix read on its upper triangle), on the exact
    gradient and on update_solution (src/tsne/mod.rs:423-451)."""
    X, _ = blobs(400, 10, 4, 13)
    X = X.astype(dtype)
    rng = np.random.default_rng(14)
    y0 = rng.normal(0.0, 1e-2, size=(400, 2)).astype(dtype)
    g, o = _exact_pair(gpu, oracle, X, variant, dtype, 3, 20.0, y0)
    ge = g.embedding().reshape(-1, 2).astype(np.float64) - y0
    oe = o.embedding().reshape(-1, 2).astype(np.float64) - y0
    assert rel_l2(ge, oe) < TOL[dtype] * 10
    assert abs(g.kl_divergence() - o.kl_divergence()) / o.kl_divergence() < TOL[dtype] * 10


@pytest.mark.parametrize("dtype,n", [(np.float32, 1000), (np.float64, 500)])
def test_exact_fit_final_kl_within_one_percent(gpu, oracle, dtype, n):
    """A full exact fit (1,000 epochs, reference defaults, perplexity 30) from
    the same initial embedding: final KL within 1 % of the oracle's."""
    # 10 overlapping clusters: final KL near 0.59, where the oracle's own
    # spread over initial embeddings 1e-6 apart is 0.2 %
    X, _ = blobs(n, 20, 10, 15, spread=3.0)
    X = X.astype(dtype)
    rng = np.random.default_rng(16)
    y0 = rng.normal(0.0, 1e-2, size=(n, 2)).astype(dtype)
    g, o = _exact_pair(gpu, oracle, X, "sqeuclidean", dtype, 1000, 30.0, y0)
    gk, ok = g.kl_divergence(), o.kl_divergence()
    assert np.isfinite(gk) and ok > 0
    assert abs(gk - ok) / ok < 0.01, (gk, ok)


def _update_inputs(dtype, n=4096, D=2, seed=17):
    rng = np.random.default_rng(seed)
    y = rng.normal(0.0, 5.0, size=(n, D)).astype(dtype)
    pos = rng.normal(0.0, 1e-3, size=(n, D)).astype(dtype)
    neg = rng.normal(0.0, 1e-1, size=(n, D)).astype(dtype)
    uy = rng.normal(0.0, 1e-2, size=(n, D)).astype(dtype)
    gains = rng.uniform(0.005, 3.0, size=(n, D)).astype(dtype)
    # Signed zeros, in every combination with the other operand's sign:
    # g = pos - neg * inv_z is -0 for (pos, neg) = (-0, +0) and +0 for
    # (+0, +0); u = +0 (the first epoch) and u = -0.
    g_cases = [(-0.0, 0.0), (0.0, 0.0), (None, None)]
    u_cases = [0.0, -0.0, None]
    k = 0
    for gp in g_cases:
        for u in u_cases:
            for _ in range(16):
                i, a = divmod(k, D)
                if gp[0] is not None:
                    pos[i, a], neg[i, a] = gp
                if u is not None:
                    uy[i, a] = u
                k += 1
    # gains below the floor after the decrease
    gains[200:260] = dtype(0.011)
    return y, pos, neg, uy, gains


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("lr,momentum,inv_z", [(200.0, 0.5, 1e-3), (20833.333, 0.8, 3.7e-7)])
def test_update_matches_gradient_step_and_zero_mean(gpu, oracle, dtype, lr, momentum, inv_z):
    """bhtsne_update against gradient_descent_step + zero_mean: gains and
    velocities bit for bit (the same per-element operations in the same
    order, Rust signum on signed zeros), positions up to the rounding of the
    mean (summed in FP64 on the device, sequentially in T by the oracle)."""
    y, pos, neg, uy, gains = _update_inputs(dtype)
    gy, guy, gg = gpu.update(y, pos, neg, uy, gains, lr, momentum, inv_z)
    oy, ouy, og = oracle.gradient_step(y, pos, neg, uy, gains, lr, momentum, inv_z)
    oy = oracle.zero_mean(oy)
    assert np.array_equal(gg, og)
    assert np.array_equal(guy.view(np.uint8), ouy.view(np.uint8)), "velocities differ (signed zeros included)"
    eps = np.finfo(dtype).eps
    scale = np.abs(oy).max()
    assert np.max(np.abs(gy.astype(np.float64) - oy)) <= 64 * eps * scale
    # The signum rule itself, restated: signs that differ add 0.2 (g = -0
    # against u = +0 counts as differing), equal signs scale by 0.8.
    g0 = pos - neg * dtype(inv_z)
    sg = np.copysign(1.0, g0)
    su = np.copysign(1.0, uy)
    expect = np.where(sg != su, gains + dtype(0.2), gains * dtype(0.8))
    expect = np.maximum(expect, dtype(0.01)).astype(dtype)
    assert np.array_equal(gg, expect)
