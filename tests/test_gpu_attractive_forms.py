"""The attractive pass over row tasks against the oracle's edge forces
(`compute_edge_forces`, src/tsne/arena.rs:398-427) on CSR matrices of chosen
row lengths: rows longer than a task (partial sums added in task order),
rows of a few entries, empty rows, D = 1..7, f32 and f64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def random_csr(n, lengths, seed, dtype):
    rng = np.random.default_rng(seed)
    rows = np.zeros(n + 1, np.uint64)
    rows[1:] = np.cumsum(lengths)
    nnz = int(rows[-1])
    cols = rng.integers(0, n, size=nnz).astype(np.uint32)
    vals = (rng.random(nnz) / nnz).astype(dtype)
    return rows, cols, vals


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("D", [1, 2, 3, 7])
def test_long_and_short_rows(gpu, oracle, dtype, D):
    """Rows of 8 to 1,500 entries (many take two or three tasks; one a dozen)
    and an entry count that is not a multiple of 128."""
    n = 3000
    rng = np.random.default_rng(40 + D)
    lengths = rng.integers(8, 300, size=n)
    lengths[17] = 1500
    lengths[-1] = 9
    rows, cols, vals = random_csr(n, lengths, 41 + D, dtype)
    assert int(rows[-1]) % 128 != 0
    y = rng.normal(0, 3.0, size=(n, D)).astype(dtype)
    method = gpu.METHOD_FIT_SNE if D == 1 else gpu.METHOD_BARNES_HUT  # Barnes-Hut covers D 2..7
    pos, _, _ = gpu.gradient(method, y, rows, cols, vals, theta=0.5)
    opos = oracle.edge_forces(y, rows, cols, vals)
    assert rel_l2(pos, opos) < (1e-5 if dtype == np.float32 else 1e-12)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_rows_of_exactly_eight(gpu, oracle, dtype):
    """Every row exactly 8 entries: most lanes of each task idle."""
    n = 1024
    rows, cols, vals = random_csr(n, np.full(n, 8), 7, dtype)
    assert int(rows[-1]) % 128 == 0
    y = np.random.default_rng(8).normal(0, 2.0, size=(n, 2)).astype(dtype)
    pos, _, _ = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
    opos = oracle.edge_forces(y, rows, cols, vals)
    assert rel_l2(pos, opos) < (1e-5 if dtype == np.float32 else 1e-12)


def test_short_and_empty_rows(gpu, oracle):
    """Rows of 0 to 39 entries; an empty row's force is zero."""
    n = 2000
    rng = np.random.default_rng(9)
    lengths = rng.integers(0, 40, size=n)
    lengths[3] = 0
    rows, cols, vals = random_csr(n, lengths, 10, np.float32)
    y = rng.normal(0, 2.0, size=(n, 2)).astype(np.float32)
    pos, _, _ = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
    opos = oracle.edge_forces(y, rows, cols, vals)
    assert rel_l2(pos, opos) < 1e-5
    assert np.all(pos[3] == 0)

