"""The two forms of the tensor-core kNN candidate pass: the resident form
(query tile in tensor memory, candidate tiles split in advance and streamed by
bulk copies; rows of at most 128 dimensions) and the staged form (producer
warps split both tiles for every candidate tile; any width). Both compute the
same 3xTF32 products in the same order, so they keep the same candidates and
thresholds: the same rows fail the certificate, and the neighbour lists are
brute force's either way."""
import os

import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def _manifold(n, dim, seed, shift):
    """n points uniform in a 10 x 10 x 10 cube, embedded isometrically in dim
    dimensions and moved by `shift` along every axis: neighbour counts grow
    with the cube of the radius, and |q|^2 grows with the shift."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(dim, 3)))
    return (rng.uniform(0.0, 10.0, size=(n, 3)) @ Q.T + shift)


def _knn(gpu, X, k, staged):
    from bhtsne_gb300 import _lib as L
    old = os.environ.get("BHTSNE_KNN_TC_STAGED")
    os.environ["BHTSNE_KNN_TC_STAGED"] = "1" if staged else "0"
    try:
        idx, dist = gpu.knn_euclidean(X, k)
        return idx, dist, L.default_context().knn_fallback_rows()
    finally:
        if old is None:
            del os.environ["BHTSNE_KNN_TC_STAGED"]
        else:
            os.environ["BHTSNE_KNN_TC_STAGED"] = old


@pytest.mark.parametrize("n,dim,k,spread", [(20000, 128, 90, 10.0), (4099, 40, 30, 1.0), (3000, 16, 90, 0.5),
                                             (1000, 5, 20, 2.0)])
def test_resident_form_matches_staged_form(gpu, oracle, n, dim, k, spread):
    X, _ = blobs(n, dim, 12, 300 + dim, spread=spread)
    ri, rd, rf = _knn(gpu, X, k, staged=False)
    si, sd, sf = _knn(gpu, X, k, staged=True)
    assert rf == sf
    assert np.array_equal(ri, si)
    assert np.array_equal(rd, sd)
    if n <= 5000:
        oi, od = oracle.knn(X, k)
        assert np.array_equal(ri, oi)
        assert np.array_equal(rd, od)


def test_staged_form_wide_rows_exact(gpu, oracle):
    """Rows of 129-256 dimensions (here 200) always take the staged form."""
    X, _ = blobs(2500, 200, 6, 9, spread=2.0)
    gi, gd = gpu.knn_euclidean(X, 60)
    oi, od = oracle.knn(X, 60)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


def test_resident_form_tail_tile_and_duplicates(gpu, oracle):
    """n = 128 m + 1 (a last tile of one row) with every point duplicated:
    exact ties across the tile boundary."""
    base, _ = blobs(577, 24, 4, 5, spread=3.0)
    X = np.concatenate([base, base[:576]])
    assert len(X) == 9 * 128 + 1
    gi, gd = gpu.knn_euclidean(X, 45)
    oi, od = oracle.knn(X, 45)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


@pytest.mark.parametrize("rescan", ["1", "0"])
def test_certificate_failures_recomputed_exactly(gpu, oracle, rescan):
    """Points away from the origin: |q|^2 is large next to the gap between the
    30th and the 128th candidate, so the candidate pass's error bound fails the
    certificate on most rows. With the
    bounded re-scan those rows take every candidate within their bound and
    re-rank it exactly (the rows whose list overflows take the brute force);
    without it (BHTSNE_KNN_RESCAN=0) they all take the brute force, whose
    candidate range (12,000 points) is split in two slices and merged. Both
    equal the oracle's brute force."""
    from bhtsne_gb300 import _lib as L
    X = _manifold(12000, 64, 21, 20.0).astype(np.float32)
    old = os.environ.get("BHTSNE_KNN_RESCAN")
    os.environ["BHTSNE_KNN_RESCAN"] = rescan
    try:
        gi, gd = gpu.knn_euclidean(X, 30)
    finally:
        if old is None:
            del os.environ["BHTSNE_KNN_RESCAN"]
        else:
            os.environ["BHTSNE_KNN_RESCAN"] = old
    ctx = L.default_context()
    failed, brute = ctx.knn_fallback_rows(), ctx.knn_brute_rows()
    assert failed > 100
    if rescan == "0":
        assert brute == failed
    else:
        assert brute < failed
    oi, od = oracle.knn(X, 30)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)


def test_bounded_rescan_f64(gpu, oracle):
    """The same rows in f64: the candidate pass runs on an f32 copy, the
    re-scan's lists are re-ranked in f64."""
    from bhtsne_gb300 import _lib as L
    X = _manifold(9000, 48, 22, 20.0).astype(np.float64)
    gi, gd = gpu.knn_euclidean(X, 30)
    ctx = L.default_context()
    assert ctx.knn_fallback_rows() > 100 and ctx.knn_brute_rows() < ctx.knn_fallback_rows()
    oi, od = oracle.knn(X, 30)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)
