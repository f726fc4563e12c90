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
    L.host_sum4_int.restype = C.c_double
    L.host_sum4_int.argtypes = [C.c_void_p, C.c_int]
    L.host_div_int.restype = C.c_double
    L.host_div_int.argtypes = [C.c_double, C.c_uint32]
    L.host_add_rn.restype = C.c_double
    L.host_add_rn.argtypes = [C.c_double, C.c_double]
    L.host_weight_ff.restype = C.c_int
    L.host_weight_ff.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_float)]
    L.host_weight_exact.restype = C.c_float
    L.host_weight_exact.argtypes = [C.c_double, C.c_double]
    L.host_units_dbl.restype = C.c_double
    L.host_units_dbl.argtypes = [C.c_uint64, C.c_int32]
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


def test_integer_addition(host):
    """ts_add_rn equals IEEE double addition (non-negative operands)."""
    rng = np.random.default_rng(10)
    a = np.concatenate([rng.random(100000) * 8.0, 2.0 ** rng.integers(-40, 14, 50000) * rng.random(50000)])
    b = np.concatenate([rng.random(100000) * 8.0, 2.0 ** rng.integers(-40, 14, 50000) * rng.random(50000)])
    a[:1000] = 0.0
    for x, y in zip(a, b):
        assert host.host_add_rn(float(x), float(y)) == float(x) + float(y), (x, y)
    # ties: y exactly half an ulp of x, and odd / even x
    for t in range(20000):
        x = float(rng.integers(1 << 52, 1 << 53)) * 2.0 ** int(rng.integers(-60, 0))
        y = math.ulp(x) / 2 * float(rng.integers(1, 4))
        assert host.host_add_rn(x, y) == x + y, (x, y)


def test_integer_division(host):
    """ts_div_int_rn(s, n) equals IEEE s / n for the mean's divisors."""
    rng = np.random.default_rng(12)
    s = np.concatenate([rng.random(100000) * 4096.0, 2.0 ** rng.integers(-40, 13, 50000) * rng.random(50000)])
    for i, x in enumerate(s):
        n = int(rng.integers(1, 1025)) if i % 2 else 4 * int(rng.integers(1, 257))
        assert host.host_div_int(float(x), n) == float(x) / n, (x, n)
    assert host.host_div_int(0.0, 200) == 0.0


def test_integer_sum4(host):
    """The 4x-duplicated in-order sum through ts_add4_rn equals the f64 chain."""
    rng = np.random.default_rng(11)
    for t in range(4000):
        n = int(rng.integers(1, 257))
        if t % 3 == 0:
            d = rng.random(n) * 4.0
        elif t % 3 == 1:
            W, H = int(rng.integers(8, 16385)), int(rng.integers(8, 16385))
            d = _distances(rng, n, W, H)
        else:  # grid-aligned values that produce exact ties
            base = float(rng.integers(1, 1 << 20)) * 2.0 ** -40
            d = np.array([base * (1 + float(rng.integers(0, 8)) / 8) for _ in range(n)])
        d[rng.random(n) < 0.05] = 0.0
        ref = 0.0
        for v in d:
            for _ in range(4):
                ref += float(v)
        got = host.host_sum4_int(d.ctypes.data, n)
        assert got == ref, (t, got, ref)


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


def _chain_mean(ds):
    """get_distances_to_k_neighs (ms.rs:405-425): the 4x-duplicated list
    summed in order with f64 adds, divided by its length."""
    s = 0.0
    for d in ds:
        s += d
        s += d
        s += d
        s += d
    return s / (4 * len(ds))


def _dists(W, H, px, py, pts):
    x2, y2 = px / W, py / H
    out = []
    for x, y in pts:
        dx, dy = x / W - x2, y / H - y2
        out.append(dx * dx + dy * dy)  # fma(dx, dx, dy*dy): both products are exact here
    return out


@pytest.mark.parametrize("W,H", [(512, 512), (256, 256), (1024, 64), (16384, 16384)])
def test_power_of_two_distance_sums_are_exact(W, H):
    """For power-of-two output sides the walk and the exhaustive k-NN sum a
    distance list in warp order instead of the reference's in-order chain
    (SessionDev::exact_sum): every distance is an integer multiple of
    1/max(W,H)^2 and no partial sum needs more than 53 bits, so both orders
    give the same double, and so the same mean."""
    import random

    rng = random.Random(W * 7 + H)
    for _ in range(300):
        k = rng.choice([1, 8, 20, 50, 256])
        px, py = rng.randrange(W), rng.randrange(H)
        # points anywhere in the plane the tree spans (tiling mirrors lie in [-W, 2W) x [-H, 2H))
        pts = [(rng.randrange(-W, 2 * W), rng.randrange(-H, 2 * H)) for _ in range(k)]
        ds = _dists(W, H, px, py, pts)
        order = list(range(k))
        rng.shuffle(order)
        tree = 0.0
        for i in order:
            tree += ds[i]
        assert 4.0 * tree / (4 * k) == _chain_mean(ds)


def test_non_power_of_two_sums_can_round():
    """The same shortcut would be wrong for other sizes: the distances are
    then inexact doubles and the order of the adds changes the sum."""
    import random

    rng = random.Random(5)
    W = H = 300
    differ = 0
    for _ in range(300):
        k = 50
        px, py = rng.randrange(W), rng.randrange(H)
        pts = [(px + rng.randrange(-9, 10), py + rng.randrange(-9, 10)) for _ in range(k)]
        ds = _dists(W, H, px, py, pts)
        tree = 0.0
        for d in reversed(ds):
            tree += d
        differ += 4.0 * tree / (4 * k) != _chain_mean(ds)
    assert differ > 0


def test_units_distances_and_means(host):
    """Outputs whose sides are powers of two: a sum of distances is
    units * 2^qe, built from the integer exactly (ts_units_bits), and the
    mean RN(4 sum / 4n) comes from integer division (ts_div_int_rn) bit for
    bit, as the k-NN kernels compute it (exact_mean)."""
    rng = np.random.default_rng(11)
    for _ in range(20000):
        qe = -2 * int(rng.integers(1, 17))
        units = int(rng.integers(0, 1 << int(rng.integers(1, 53))))
        d = host.host_units_dbl(units, qe)
        assert d == math.ldexp(float(units), qe) and float(units) == units
        n = int(rng.integers(1, 300))
        ref = (4.0 * d) / float(4 * n)
        got = host.host_div_int(d, n)
        assert np.float64(got).view(np.uint64) == np.float64(ref).view(np.uint64), (units, qe, n)

