"""The double-word arithmetic of csrc/dword.cuh, compiled as host code and checked against
long-double references on random operands (including near-cancelling ones): worst errors in units
of u^2 = 2^-48 against the bounds the kernels rely on."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "sayram-2d_gb300", "csrc")

BOUNDS = {  # published bounds (Joldes, Muller, Popescu 2017) or the bound stated in dword.cuh
    "add": 3.0, "add_same_same_sign": 3.0, "add_same_any_sign_vs_magnitudes": 3.0, "mul": 4.0,
    "rcp": 6.0, "div": 8.0, "fma_vs_magnitudes": 6.0, "add_f": 2.0, "mul_f": 2.0, "dot2_vs_magnitudes": 6.0,
}


def test_dword_error_bounds(tmp_path):
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "dword_check")
    # -ffp-contract=off: every product and sum rounded separately, as the algorithms assume
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", cuda_inc,
                    os.path.join(HERE, "dword", "dword_check.cc"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    worst = {ln.split()[0]: float(ln.split()[1]) for ln in out.strip().splitlines()}
    assert set(worst) == set(BOUNDS)
    for k, b in BOUNDS.items():
        assert worst[k] <= b, (k, worst[k], b)


def test_integer_conversions_match_the_fp64_ones(tmp_path):
    """dw_from_double_int / dw_to_double_int (the layout transforms' conversions) give the bits of
    dw_from_double / dw_to_double on every binary exponent of the double range, on rounding ties
    with carries into the exponent, on special values and on arbitrary float pairs."""
    cxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not cxx or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "convert_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", cuda_inc,
                    os.path.join(HERE, "dword", "convert_check.cc"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "from_double_mismatches 0 to_double_mismatches 0" in out.stdout
