"""The allocation-free Barnes-Hut entry point (bhtsne_bh_repulsion_noalloc).

It exists for callers that cannot allocate device memory: code recording into
a CUDA stream capture, hosts that hand the library a fixed device budget, and
loops where an allocation could synchronise the device. Through the C ABI it
must give the same forces and Z as the allocating entry point
(bhtsne_gradient, Barnes-Hut), on two calls in a row (the shared scratch keeps
the first call's contents when the second starts). This file sorts last so
that a failure here stops a -x run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    import bhtsne_gb300 as bg
    lib = bg.load()
    rng = np.random.default_rng(2024)
    dev = torch.device("cuda:0")
    calls = 0
    for n, scale in ((20000, 4.0), (6000, 0.5), (20000, 4.0)):
        y = rng.normal(0.0, scale, size=(n, 2)).astype(np.float32)
        # the allocating entry point (host buffers)
        rows = np.zeros(n + 1, np.uint64)
        _, neg_ref, z_ref = bg.gradient(bg.METHOD_BARNES_HUT, y, rows, np.zeros(0, np.uint32),
                                        np.zeros(0, np.float32), theta=0.5)
        # the allocation-free one (device buffers owned by the caller)
        y_d = torch.from_numpy(y).to(dev)
        neg_d = torch.zeros((n, 2), dtype=torch.float32, device=dev)
        z_d = torch.zeros(1, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.bhtsne_bh_repulsion_noalloc(C.c_void_p(y_d.data_ptr()), n, 0.5, C.c_void_p(neg_d.data_ptr()),
                                             C.c_void_p(z_d.data_ptr()), None)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0
        if calls > 0:
            # after the first call (which may load the library's device code and
            # its fixed array), a call leaves the device's free memory unchanged
            assert free_after == free_before, (free_before, free_after)
        calls += 1
        neg = neg_d.cpu().numpy()
        z = float(z_d.cpu().numpy()[0])
        assert rel_l2(neg, neg_ref) < 1e-4
        assert abs(z - z_ref) / z_ref < 1e-4


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    import bhtsne_gb300 as bg
    lib = bg.load()
    dev = torch.device("cuda:0")
    y_d = torch.zeros((4, 2), dtype=torch.float32, device=dev)
    neg_d = torch.zeros((4, 2), dtype=torch.float32, device=dev)
    z_d = torch.zeros(1, dtype=torch.float64, device=dev)
    rc = lib.bhtsne_bh_repulsion_noalloc(C.c_void_p(y_d.data_ptr()), 32769, 0.5, C.c_void_p(neg_d.data_ptr()),
                                         C.c_void_p(z_d.data_ptr()), None)
    assert rc == bg._lib.EINVAL
