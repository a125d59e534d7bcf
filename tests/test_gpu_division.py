"""The AMAZE weights are computed in registers: 1/(1+gradient) by a reciprocal estimate and one
Newton-Raphson step (dev::rcp_small_int), the normalisation by one remainder correction per
quotient (dev::weight_quotients).  This test compares them with CUDA's correctly rounded
operations exhaustively: every reciprocal up to 3 * 65535 + 1, and every weight pair bit depths up
to 12 can produce (12287^2 pairs)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_weight_quotients_equal_ieee_division_exhaustively(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "div_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", os.path.join(HERE, "gpu_kernels", "div_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe, "12"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" 0 mismatches") == 2


def test_jpeg_quotients_equal_ieee_division_exhaustively(tmp_path):
    """The JPEG quantiser division (reciprocal product plus one residual correction) against
    __fdiv_rn for every float in [0.5, 2048) and every quantiser 1..255."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "jpeg_quant_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", os.path.join(HERE, "gpu_kernels", "jpeg_quant_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
