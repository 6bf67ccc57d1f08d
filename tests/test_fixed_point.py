"""The integer-only f32 <-> int64 conversions of the FIt-SNE fixed-point
charges round to nearest even and saturate like the IEEE conversions (so the
spread and the charge grids hold the same values as with the hardware
conversions). Host-only: compiled with nvcc and run on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fixed_point_conversions_round_to_nearest_even(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "fixed_point_conversions")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "bhtsne_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "fixed_point_conversions.cu")], check=True,
                   capture_output=True, timeout=300)
    r = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
