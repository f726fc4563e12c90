"""Weight primitives on the host (ts_common.h built with g++):
  - ts_exp64 equals the oracle's exp bit for bit and stays within 2 ulp of
    libm's exp;
  - the Markstein division equals IEEE division;
  - the double-f32 weight, whenever it decides, equals the exact f64 weight.
"""
import ctypes as C
import math
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hm") / "host_math.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "texture-synthesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cuda", "host_math.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    L.host_exp.restype = C.c_double
    L.host_exp.argtypes = [C.c_double]
    L.host_div.restype = C.c_double
    L.host_div.argtypes = [C.c_double, C.c_double]
    L.host_weight_ff.restype = C.c_int
    L.host_weight_ff.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_float)]
    L.host_weight_exact.restype = C.c_float
    L.host_weight_exact.argtypes = [C.c_double, C.c_double]
    return L


def test_exp_matches_oracle_and_libm(host, oracle):
    rng = np.random.default_rng(5)
    xs = np.concatenate([-700 * rng.random(20000), -16 * rng.random(60000) ** 2, [0.0, -0.0, -700.0, -1e-300]])
    worst = 0.0
    for x in xs:
        a = host.host_exp(float(x))
        b = oracle.lib().tso_exp_export(float(x))
        assert np.float64(a).view(np.uint64) == np.float64(b).view(np.uint64), x
        ref = math.exp(float(x))
        if ref > 1e-300:
            worst = max(worst, abs(a - ref) / math.ulp(ref))
    assert worst <= 2.0, worst
    assert math.isnan(host.host_exp(float("nan")))


def test_markstein_division(host):
    rng = np.random.default_rng(6)
    a = rng.random(200000) * 8.0
    b = rng.random(200000) * 2.0 + 1e-12
    for x, y in zip(a, b):
        assert host.host_div(float(x), float(y)) == float(x) / float(y)


def _distances(rng, n, W, H):
    """Distances as the weights see them: fma(dx, dx, dy*dy) of normalised
    lattice offsets (computed like ms.rs:410-415)."""
    px, py = rng.integers(0, W), rng.integers(0, H)
    ox = rng.integers(-40, 41, n)
    oy = rng.integers(-40, 41, n)
    out = []
    for a, b in zip(ox, oy):
        dx = (px + a) / W - px / W
        dy = (py + b) / H - py / H
        # fused multiply-add: exact rational arithmetic, one rounding
        out.append(float(Fraction(dx) * Fraction(dx) + Fraction(dy * dy)))
    return np.array(out, np.float64)


def test_fast_weight_matches_exact(host):
    rng = np.random.default_rng(8)
    w = C.c_float()
    decided = 0
    total = 0
    for t in range(400):
        W, H = int(rng.integers(16, 4097)), int(rng.integers(16, 4097))
        d = _distances(rng, 50, W, H)
        mean = 0.0
        for v in d:
            for _ in range(4):
                mean += float(v)
        mean /= 200.0
        for v in d:
            total += 1
            exact = host.host_weight_exact(float(v), mean)
            if host.host_weight_ff(float(v), mean, C.byref(w)):
                decided += 1
                assert np.float32(w.value).view(np.uint32) == np.float32(exact).view(np.uint32), (v, mean)
    assert decided > 0.99 * total, (decided, total)
    # all distances zero: 0 / 0 is NaN in the reference; the fast path defers
    assert host.host_weight_ff(0.0, 0.0, C.byref(w)) == 0
    assert math.isnan(host.host_weight_exact(0.0, 0.0))
