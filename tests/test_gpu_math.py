"""The f64 primitives behind the neighbour weights, on the GPU.

The weights kernel divides by the mean through a reciprocal and Markstein's
correction, and exponentiates with the table-driven ts_exp64 of
ts_common.h; the oracle divides with IEEE division and runs the same exp
algorithm on the host.  This test compiles tests/cuda/math_check.cu against
the product header and checks, over 4M inputs:
  - the Markstein quotient equals __ddiv_rn bit for bit (and the host's /),
  - ts_exp64 on the device equals ts_exp64 on the host bit for bit,
  - ts_exp64 is within 2 ulp of CUDA's exp(),
  - the double-f32 weight, when it decides, equals the exact f64 weight
    (and decides for more than 99.9% of inputs),
  - the integer mean (ts_add4_rn, ts_div_int_rn) equals the __dadd_rn chain
    divided by __ddiv_rn.
"""
import json
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_weight_math(tmp_path):
    exe = str(tmp_path / "math_check")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--fmad=false",
                    "-Xcompiler", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "texture-synthesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cuda", "math_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    assert r["div_mismatch"] == 0, r
    assert r["host_div_mismatch"] == 0, r
    assert r["exp_host_device_mismatch"] == 0, r
    assert r["exp_over_2ulp"] == 0, r
    assert r["weight_mismatch"] == 0, r
    assert r["weight_undecided"] < r["n"] // 1000, r
    assert r["mean_mismatch"] == 0, r
