"""The FP32 -> FP64 widening of the Krylov kernels (vfs::widen, integer
pipe) is compiled for the host from the same header and compared with the
compiler's conversion over a stride of all 2^32 float bit patterns plus every
special class (zeros, subnormals, infinities, quiet and signalling NaNs)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_widen_matches_hardware_conversion(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "widen_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "vfs_v3p2_gb300", "csrc"),
                    os.path.join(HERE, "native", "widen_check.cu"), "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe, "257"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
