"""Integer-pipe float<->double conversions and the short-chain FP64 helpers
(finitevolume_gb300/csrc/fpconv.cuh).

The FP32-flux kernels widen face fluxes and round the state with these
routines instead of the hardware conversions (which issue on GB300's scarce
FP64 pipe).  They must agree with the hardware bit for bit: exhaustively
for float -> double, and on 2^31 double patterns weighted towards the
rounding and range boundaries for double -> float.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_integer_conversions_match_hardware(gpu, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "fpconv_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
                    os.path.join(ROOT, "finitevolume_gb300", "csrc"), os.path.join(ROOT, "tests", "cuda", "fpconv_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "f2d_mismatch 0 d2f_mismatch 0" in r.stdout


@pytest.mark.gpu
def test_fp64_reciprocal_within_an_ulp(gpu, tmp_path):
    """fvconv::rcp_nr3, the FP64 reciprocal of the second-order kernels
    (limiter quotient, local time step, 1/rho of the primitive copy): within
    one ulp of the IEEE reciprocal on 2^30 inputs (equal to it on at least
    99%), and the IEEE result itself outside the float normal range."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "rcp_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
                    os.path.join(ROOT, "finitevolume_gb300", "csrc"), os.path.join(ROOT, "tests", "cuda", "rcp_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    f = r.stdout.split()
    vals = dict(zip(f[0:8:2], map(int, f[1:8:2])))
    assert vals["rcp_bad"] == 0 and vals["rcp_max_ulp"] <= 1
    assert vals["rcp_inexact"] <= vals["rcp_checked"] // 100, r.stdout


@pytest.mark.gpu
def test_pow_near1_matches_library_pow(gpu, tmp_path):
    """fvconv::pow_near1 (the boundary density power of the characteristic
    farfield in the persistent first-order kernel): within 8 ulps of the
    library pow for bases in [7/8, 9/8], pow itself outside, on 2^26
    pseudo-random bases and eight exponents (2/(g-1) for g = 1.1 .. 1.67
    among them)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "pow_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I",
                    os.path.join(ROOT, "finitevolume_gb300", "csrc"), os.path.join(ROOT, "tests", "cuda", "pow_check.cu"),
                    "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    f = r.stdout.split()
    vals = dict(zip(f[0:8:2], map(int, f[1:8:2])))
    assert vals["pow_bad"] == 0, r.stdout
    assert vals["pow_max_ulp"] <= 8, r.stdout
