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


def test_sliced_certified_fallback_exact(gpu, oracle):
    """Points far from the origin: |q|^2 dwarfs the neighbour gaps, so the
    candidate pass's error bound fails the certificate on most rows, and the
    fallback (12,000 points: its candidate range split in two slices, merged)
    recomputes them exactly."""
    from bhtsne_gb300 import _lib as L
    X, _ = blobs(12000, 64, 10, 21, spread=2.0)
    X = (X + np.float32(1000.0)).astype(np.float32)
    gi, gd = gpu.knn_euclidean(X, 30)
    assert L.default_context().knn_fallback_rows() > 1000
    oi, od = oracle.knn(X, 30)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gd, od)
