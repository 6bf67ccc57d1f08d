"""bench.py on the CPU: seeded input generators of the configured shapes, the
within-cluster kNN that feeds the CPU arm (the clusters of the 1M-point mixture
are far apart, so it is the global kNN), and the JSON line of the reference arm
(`--impl reference`, which times the oracle) at a small N."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_workload_generators_are_seeded_and_shaped():
    a, la = bench.make_workload(2000)
    b, lb = bench.make_workload(2000)
    assert a.dtype == np.float32 and a.shape == (2000, 128) and a.flags["C_CONTIGUOUS"]
    assert np.array_equal(a, b) and np.array_equal(la, lb)
    assert la.min() >= 0 and la.max() < 100
    assert bench.make_c1_workload(500).shape == (500, 50)
    c2 = bench.make_c2_workload(700)
    assert c2.shape == (700, 20) and c2.dtype == np.float32
    assert np.array_equal(c2, bench.make_c2_workload(700))


def test_within_cluster_knn_is_the_global_knn(oracle):
    X, lab = bench.make_workload(6000)
    idx, dist = bench.within_cluster_knn(X, lab, 30)
    oi, od = oracle.knn(X, 30)
    same = np.mean([set(a) == set(b) for a, b in zip(idx.astype(np.int64), oi.astype(np.int64))])
    assert same > 0.99, same
    assert np.allclose(np.sort(dist, 1), od, rtol=1e-3, atol=1e-3)


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "20000",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "epochs/s" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] >= 3 and line["higher_is_better"] is True  # W >= 3 enforced
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"] == "bh2d_1M_d128" and line["config"]["n_points"] == 20000
    # the same config object the GPU arm prints, window included (250 burn-in
    # + 3 warm-up epochs, then the 2 timed ones)
    from types import SimpleNamespace
    assert line["config"] == bench.workload_config(SimpleNamespace(n=20000, burn_in=250, warmup=3, steps=2), 1)
    assert "epochs 253-254" in line["config"]["window"]


def test_interaction_count_at_tiny_theta_is_all_pairs(oracle):
    """With theta -> 0 every internal cell is opened, so each point interacts
    with every other leaf once: n (n - 1) accepted cells."""
    rng = np.random.default_rng(4)
    y = rng.normal(size=(400, 2)).astype(np.float32)
    vis, inter = oracle.bh_interactions(y, 1e-6)
    assert inter == 400 * 399 and vis > inter
    vis5, inter5 = oracle.bh_interactions(y, 0.5)
    assert 0 < inter5 < inter and inter5 <= vis5


def test_cpu_leg_counts_barnes_hut_work(oracle):
    from types import SimpleNamespace
    X, _ = bench.make_workload(6000)
    idx, dist = oracle.knn(X, 30)
    t = oracle.TSNE(6000).perplexity(10.0).epochs(0).seed(3)
    t.barnes_hut_with_neighbors(0.5, idx, dist)
    rows, cols, vals, perp = t.affinities()
    aff = SimpleNamespace(rows=rows, columns=cols, values=vals, perplexity=perp)
    y0 = t.embedding().reshape(6000, 2)
    out = bench.cpu_baseline_sample(aff, y0, 2, count_at=y0)
    assert out["kind"] == "port" and out["value"] > 0
    w = out["bh_work_per_epoch"]
    assert 0 < w["interactions"] <= w["theta_tests"]
