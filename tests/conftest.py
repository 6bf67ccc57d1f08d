"""Shared fixtures. GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running (full-size) case")


def lcg_samples(n, dim, state):
    """The reference tests' LCG (src/test.rs:973-982): (state >> 33) / u32::MAX - 0.5 in f32."""
    out = np.empty(n * dim, np.float32)
    s = state & 0xFFFFFFFFFFFFFFFF
    inv = np.float32(4294967295.0)
    for i in range(n * dim):
        s = (s * 6364136223846793005 + 1442695040888963407) & 0xFFFFFFFFFFFFFFFF
        out[i] = np.float32(np.float32(s >> 33) / inv) - np.float32(0.5)
    return out.reshape(n, dim)


def blobs(n, dim, k, seed, spread=10.0):
    """Seeded isotropic Gaussian mixture (equal weights, centres ~ N(0, spread^2 I))."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, spread, size=(k, dim))
    lab = rng.integers(0, k, size=n)
    X = centres[lab] + rng.normal(size=(n, dim))
    return X.astype(np.float32), lab


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    import bhtsne_gb300 as bg
    return bg
