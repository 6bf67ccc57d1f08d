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
