"""The single-pass radix sort (decoupled look-back, from 131,072 keys) against
the three-kernel passes: both are stable LSD sorts, so the Barnes-Hut tree
built from either permutation, and the repulsion from it, are the same bit for
bit. Sizes include a last tile that is not full, 128-bit codes (D = 5) and
several sorts in a row (the look-back words are cleared between sorts)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def clustered(n, D, seed):
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 40.0, size=(64, D))
    return (centres[rng.integers(0, 64, n)] + rng.normal(size=(n, D)) * 2.0).astype(np.float32)


@pytest.mark.parametrize("n,D", [(131072, 2), (200001, 2), (300000, 3), (140000, 5)])
def test_onesweep_matches_multipass(gpu, monkeypatch, n, D):
    y = clustered(n, D, n + D)
    rows = np.zeros(n + 1, np.uint64)
    cols, vals = np.zeros(0, np.uint32), np.zeros(0, np.float32)
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("BHTSNE_SORT_ONESWEEP", mode)
        res = []
        for rep in range(2):  # twice: the second sort reuses the look-back scratch
            _, neg, z = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
            res.append((neg.copy(), z))
        assert np.array_equal(res[0][0], res[1][0]) and res[0][1] == res[1][1]
        out[mode] = res[0]
    assert np.array_equal(out["1"][0].view(np.uint32), out["0"][0].view(np.uint32))
    assert out["1"][1] == out["0"][1]
