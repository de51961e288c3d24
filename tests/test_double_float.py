"""The double-float helpers of the fixed-point forms (codyfortran_gb300/csrc/dfloat.cuh)
on the host: tests/df_check.cu is compiled by nvcc as host code and checks
  * the FP64 -> double-float split and back (the low part rounded to 24 bits),
    and that the round trip carries no one-sided bias (mean signed relative
    error over 2e6 values below 1e-17; the earlier truncating split gave
    -1.5e-15, a drift of the state norm over long runs),
  * the integer FP64 conversion of any (hi, lo) pair against the correctly
    rounded FP64 sum: equal to it (round to nearest, ties to even), and exact
    where the sum is representable,
  * complex double-float dot products of up to 600 terms against long double
    sums: within 2^-41 of the sum of magnitudes (measured 1.9e-13, about
    2^-42.3: the operands keep 48 bits, the low parts add in FP32),
  * zero, infinity and FP32 subnormals.
The device kernels compile the same header, so the integer logic is the one
checked here.
"""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_double_float_helpers(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "df_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "df_check.cu")], check=True)
    r = json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    assert r["split_bad"] == 0
    assert r["split_rel_max"] < 2.0 ** -46
    assert r["conv_bad"] == 0 and r["conv_ulps_max"] <= 0.5
    assert r["conv_exact_cases"] > 100000 and r["conv_exact_bad"] == 0
    assert r["dot_rel_max"] < 2.0 ** -41
    assert r["specials"]
    assert abs(r["split_bias"]) < 1e-17
