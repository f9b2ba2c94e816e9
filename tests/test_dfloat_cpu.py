"""Host build of the block-floating-point residuals (afmibins_gb300/csrc/
dfloat.cuh, the FP64-state residuals of the mixed form evaluated without FP64
instructions) against exact rational arithmetic."""
import ctypes
import os
import shutil
import subprocess
from fractions import Fraction as Fr

import numpy as np
import pytest

from afmibins_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("dfloat") / "libdfloat.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    "-I", os.path.join(build.PKG, "csrc"), os.path.join(HERE, "cpp", "dfloat_host.cc"),
                    "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    dp, ip, fp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)
    L.afmib_test_helm_residual.argtypes = [ctypes.c_double, ctypes.c_double, dp, ip, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double]
    L.afmib_test_helm_residual.restype = ctypes.c_float
    L.afmib_test_lap_residual.argtypes = [ctypes.c_double, ctypes.c_double, dp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int]
    L.afmib_test_lap_residual.restype = ctypes.c_float
    L.afmib_test_split.argtypes = [ctypes.c_double, fp, fp]
    L.afmib_test_sincospi.argtypes = [ctypes.c_double, fp, fp]
    L.afmib_test_df_hi.argtypes = [ctypes.c_double]
    L.afmib_test_df_hi.restype = ctypes.c_float
    L.afmib_test_df_round.argtypes = [ctypes.c_double]
    L.afmib_test_df_round.restype = ctypes.c_float
    L.afmib_test_split_round.argtypes = [ctypes.c_double, fp, fp]
    L.afmib_test_lap_update_df.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, fp, ctypes.c_int,
                                           ctypes.c_float, ctypes.c_float, fp, fp]
    L.afmib_test_helm_update_df.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, fp, ctypes.c_int,
                                            ctypes.c_float, ctypes.c_double, ctypes.c_float, ctypes.c_double,
                                            ctypes.c_int, fp, fp]
    L.afmib_test_fixed.argtypes = [ctypes.c_longlong, ctypes.c_int, fp, fp]
    L.afmib_test_convert_mismatches.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong]
    L.afmib_test_convert_mismatches.restype = ctypes.c_longlong
    return L


def test_integer_conversion_matches_ieee_cast(lib):
    """f32_to_f64 (the integer-op widening used by the mixed form's FP64
    kernels) agrees bit for bit with the C cast on zeros, subnormals, inf,
    nan, normal values and raw bit patterns."""
    assert lib.afmib_test_convert_mismatches(2_000_000, 12345) == 0


def _arr(a, t):
    return (t * len(a))(*a)


def test_split_keeps_47_bits(lib):
    rng = np.random.default_rng(1)
    hi, lo = ctypes.c_float(), ctypes.c_float()
    for _ in range(3000):
        d = float(rng.standard_normal() * 10.0 ** rng.uniform(-20, 20))
        lib.afmib_test_split(d, ctypes.byref(hi), ctypes.byref(lo))
        assert abs((Fr(hi.value) + Fr(lo.value)) - Fr(d)) <= abs(Fr(d)) * Fr(2) ** -46
    lib.afmib_test_split(0.0, ctypes.byref(hi), ctypes.byref(lo))
    assert hi.value == 0.0 and lo.value == 0.0


def test_fixed_to_pair(lib):
    rng = np.random.default_rng(2)
    hi, lo = ctypes.c_float(), ctypes.c_float()
    for _ in range(3000):
        q = int(rng.integers(-(2 ** 61), 2 ** 61))
        E = int(rng.integers(1000, 1100))
        lib.afmib_test_fixed(q, E, ctypes.byref(hi), ctypes.byref(lo))
        exact = Fr(q) * Fr(2) ** (E - 1078)
        assert abs(Fr(hi.value) + Fr(lo.value) - exact) <= abs(exact) * Fr(2) ** -47


def _helm_cases(rng, n):
    for _ in range(n):
        off = float(0.0066 * rng.uniform(0.2, 3.0))
        x0 = float(0.3 + 0.1 * rng.standard_normal())
        nb = [float(x0 + 1e-3 * rng.standard_normal()) for _ in range(6)]
        exact_hx = Fr(x0) + Fr(off) * (sum(Fr(v) for v in nb) - 6 * Fr(x0))
        b = float(exact_hx + Fr(float(10.0 ** rng.uniform(-16, -9) * rng.choice([-1, 1]))))
        yield off, x0, nb, b


def test_helm_residual_beats_fp64_formula(lib):
    """Near convergence (|r| ~ 1e-16 .. 1e-9 against |x| ~ 0.3) the residual
    from the block arithmetic carries only the float rounding of r itself,
    below the rounding of the FP64 formula it replaces."""
    rng = np.random.default_rng(3)
    cnb = _arr([1] * 6, ctypes.c_int)
    for off, x0, nb, b in _helm_cases(rng, 2000):
        r = lib.afmib_test_helm_residual(b, x0, _arr(nb, ctypes.c_double), cnb, 6, -6, off)
        exact = Fr(b) - (Fr(x0) + Fr(off) * (sum(Fr(v) for v in nb) - 6 * Fr(x0)))
        err = abs(Fr(r) - exact)
        M = max(abs(Fr(v)) for v in [b, x0] + nb)
        # float rounding of r plus a few FP64 units of the largest value (each
        # value truncates by at most 2^-55 of it at the block's scale; the FP64
        # formula itself rounds at that order)
        assert err <= abs(exact) * Fr(2) ** -23 + M * Fr(2) ** -50, (float(err), float(exact))


def test_helm_residual_channel_wall_row(lib):
    """Wall rows of the u/w Helmholtz operator: H x = x0 + (off/3)(3 sx + 3 sz + 4 x1 - 24 x0)."""
    rng = np.random.default_rng(4)
    cnb = _arr([3, 3, 3, 3, 4], ctypes.c_int)
    for _ in range(1000):
        off = float(0.0066 * rng.uniform(0.2, 3.0))
        x0 = float(0.2 + 0.1 * rng.standard_normal())
        nb = [float(x0 + 1e-3 * rng.standard_normal()) for _ in range(5)]
        f = off / 3
        exact_hx = Fr(x0) + Fr(f) * (sum(c * Fr(v) for c, v in zip([3, 3, 3, 3, 4], nb)) - 24 * Fr(x0))
        b = float(exact_hx + Fr(1e-12))
        r = lib.afmib_test_helm_residual(b, x0, _arr(nb, ctypes.c_double), cnb, 5, -24, f)
        exact = Fr(b) - (Fr(x0) + Fr(f) * (sum(c * Fr(v) for c, v in zip([3, 3, 3, 3, 4], nb)) - 24 * Fr(x0)))
        # the wall row does not annihilate constants (row sum 1 - 8 off / 3),
        # so f Q is as large as x and carries f's pair rounding (2^-46)
        fq = abs(Fr(f) * (sum(c * Fr(v) for c, v in zip([3, 3, 3, 3, 4], nb)) - 24 * Fr(x0)))
        M = max(abs(Fr(v)) for v in [b, x0] + nb)
        bound = abs(exact) * Fr(2) ** -23 + fq * Fr(2) ** -44 + M * Fr(2) ** -50
        assert abs(Fr(r) - exact) <= bound


def test_lap_residual(lib):
    rng = np.random.default_rng(5)
    n = 256
    k2 = 16
    for _ in range(2000):
        x0 = float(1e-4 * rng.standard_normal())
        nb = [float(x0 + 1e-6 * rng.standard_normal()) for _ in range(6)]
        c = int(rng.choice([6, 5, 4]))
        m = 6 if c == 6 else c
        exact_l = Fr(n * n) * (sum(Fr(v) for v in nb[:m]) - c * Fr(x0))
        b = float(exact_l + Fr(float(rng.standard_normal() * 1e-11)))
        r = lib.afmib_test_lap_residual(b, x0, _arr(nb[:m], ctypes.c_double), m, c, k2)
        exact = Fr(b) - exact_l
        M = max([abs(Fr(b)) / (n * n)] + [abs(Fr(v)) for v in [x0] + nb[:m]])
        assert abs(Fr(r) - exact) <= abs(exact) * Fr(2) ** -23 + n * n * M * Fr(2) ** -50


@pytest.mark.parametrize("kind", ["interior", "2d", "wall"])
def test_helm_update_df(lib, kind):
    """Outer residual update of the mixed viscous solve, r - H e for an FP32
    correction e in double-float (df_helm_row), against exact rational
    arithmetic: the error stays within a few units of 2^-44 of H e's largest
    term plus 2^-46 of r, down to residuals 1e-5 of the correction."""
    rng = np.random.default_rng(6)
    f32 = lambda v: float(np.float32(v))
    nnb, k, wall = {"interior": (6, 6.0, 0), "2d": (4, 4.0, 0), "wall": (4, 8.0, 1)}[kind]
    for it in range(3000):
        off = float(10.0 ** rng.uniform(-4, 1))
        cxa = off + off / 3
        e0 = f32(10.0 ** rng.uniform(-8, 0) * rng.standard_normal())
        nb = [f32(e0 * (1 + 10.0 ** rng.uniform(-6, 0) * rng.standard_normal())) for _ in range(nnb)]
        xa = f32(e0 * (1 + 0.1 * rng.standard_normal())) if wall else 0.0
        he = Fr(e0) + Fr(off) * (sum(Fr(v) for v in nb) - Fr(k) * Fr(e0)) + (Fr(cxa) * Fr(xa) if wall else 0)
        r = float(he) * (1 + 1e-5 * rng.standard_normal())
        rh = f32(r)
        rl = f32(r - rh)
        oh, ol = ctypes.c_float(), ctypes.c_float()
        lib.afmib_test_helm_update_df(rh, rl, e0, _arr(nb, ctypes.c_float), nnb, k, off, xa, cxa, wall,
                                      ctypes.byref(oh), ctypes.byref(ol))
        exact = Fr(rh) + Fr(rl) - he
        scale = abs(Fr(e0)) + abs(Fr(off)) * (sum(abs(Fr(v)) for v in nb) + Fr(k) * abs(Fr(e0)))
        if wall:
            scale += abs(Fr(cxa) * Fr(xa))
        bound = scale * Fr(2) ** -44 + (abs(Fr(rh)) + abs(Fr(rl))) * Fr(2) ** -46
        assert abs(Fr(oh.value) + Fr(ol.value) - exact) <= bound, (it, kind)
        # the pair is normalised: hi is the float nearest to the pair
        assert oh.value == f32(Fr(oh.value) + Fr(ol.value))


@pytest.mark.parametrize("c", [6.0, 5.0, 4.0])
def test_lap_update_df(lib, c):
    """Outer residual update of the mixed pressure solve, r - L e for an FP32
    correction in double-float (df_lap_row; c = 6 interior, 5 next to a
    channel wall, 4 in 2D, missing neighbours as zeros), against exact
    rational arithmetic."""
    rng = np.random.default_rng(7)
    f32 = lambda v: float(np.float32(v))
    for it in range(3000):
        n = int(rng.choice([16, 64, 256, 96, 4096]))
        off = float(n * n)
        e0 = f32(10.0 ** rng.uniform(-10, -2) * rng.standard_normal())
        m = int(c)
        nb = [f32(e0 * (1 + 10.0 ** rng.uniform(-6, 0) * rng.standard_normal())) for _ in range(m)]
        nb += [0.0] * (6 - m)
        le = Fr(off) * (sum(Fr(v) for v in nb) - Fr(c) * Fr(e0))
        r = float(le) * (1 + 1e-5 * rng.standard_normal())
        rh = f32(r)
        rl = f32(r - rh)
        oh, ol = ctypes.c_float(), ctypes.c_float()
        lib.afmib_test_lap_update_df(rh, rl, e0, _arr(nb, ctypes.c_float), 6, c, off, ctypes.byref(oh),
                                     ctypes.byref(ol))
        exact = Fr(rh) + Fr(rl) - le
        scale = Fr(off) * (sum(abs(Fr(v)) for v in nb) + Fr(c) * abs(Fr(e0)))
        bound = scale * Fr(2) ** -44 + (abs(Fr(rh)) + abs(Fr(rl))) * Fr(2) ** -46
        assert abs(Fr(oh.value) + Fr(ol.value) - exact) <= bound, it


def test_df_hi_truncates(lib):
    """df_hi (the FP32 shadow of the velocity, by integer operations): the
    float of the double's leading 24 bits, truncated toward zero, over the
    float normal range; zero below it."""
    rng = np.random.default_rng(8)
    for _ in range(20000):
        d = float(rng.standard_normal() * 10.0 ** rng.uniform(-30, 30))
        h = lib.afmib_test_df_hi(d)
        f = float(np.float32(d))  # nearest
        # truncation: |h| <= |d|, same sign, and h is f or the float next to f toward zero
        assert abs(h) <= abs(d) and (h == 0.0 or np.sign(h) == np.sign(d))
        assert h == f or h == float(np.nextafter(np.float32(f), np.float32(0.0)))
    assert lib.afmib_test_df_hi(1e-45) == 0.0 and lib.afmib_test_df_hi(-0.0) == 0.0
    assert lib.afmib_test_df_hi(0.1) == float(np.float32(0.1)) or lib.afmib_test_df_hi(0.1) < 0.1


def test_df_round_is_nearest(lib):
    """df_round (the mixed form's FP32 velocity shadow, by integer
    operations): the float nearest to the double over the float normal range
    (the IEEE cast, except that exact ties go away from zero), carries into the
    exponent included; zero below the range."""
    rng = np.random.default_rng(9)
    for _ in range(20000):
        d = float(rng.standard_normal() * 10.0 ** rng.uniform(-30, 30))
        r = lib.afmib_test_df_round(d)
        assert r == float(np.float32(d)), d
    # exact ties: away from zero (the cast rounds to even)
    for m in (1.0 + 2.0 ** -24, 1.0 + 3.0 * 2.0 ** -24, -(1.0 + 2.0 ** -24)):
        r = lib.afmib_test_df_round(m)
        assert abs(r) > abs(m) and abs(r) - abs(m) == 2.0 ** -24
    # carry into the exponent: just below 2 rounds to 2
    assert lib.afmib_test_df_round(2.0 - 2.0 ** -30) == 2.0
    assert lib.afmib_test_df_round(1e-45) == 0.0 and lib.afmib_test_df_round(-0.0) == 0.0


def test_split_round_pair(lib):
    """df_split_round (the mixed form's velocity pair for the FP32 advection):
    hi is the nearest float, lo the rest, and hi + lo is d to 2^-46 of |d|
    (exact rationals), over the float normal range; below 2^-80, where the
    rest underflows, the truncated pair."""
    rng = np.random.default_rng(10)
    hi, lo = ctypes.c_float(), ctypes.c_float()
    for _ in range(20000):
        d = float(rng.standard_normal() * 10.0 ** rng.uniform(-25, 25))
        lib.afmib_test_split_round(d, ctypes.byref(hi), ctypes.byref(lo))
        if abs(d) >= 2.0 ** -79:
            assert hi.value == float(np.float32(d))
            assert abs(Fr(hi.value) + Fr(lo.value) - Fr(d)) <= abs(Fr(d)) * Fr(2) ** -46, d
        else:  # the rest underflows: the truncated pair, within one float ulp
            assert abs(Fr(hi.value) + Fr(lo.value) - Fr(d)) <= abs(Fr(d)) * Fr(2) ** -23, d


def test_df_sincospi_against_exact(lib):
    """df_sincospi (the mixed form's marker weights on the FP32 pipe) against
    sin(pi x) and cos(pi x) from a 40-digit Taylor evaluation, over [0, 1/2]
    including both ends and the reflection point 1/4: relative error below
    2^-44 of the larger of the two values (the weights (1 -+ S)/4, (1 +- C)/4
    then carry it as an absolute error below 2^-45)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 50
    pi = Decimal("3.14159265358979323846264338327950288419716939937510")

    def exact(x):
        t = pi * Decimal(x)
        s = c = Decimal(0)
        term_s, term_c = t, Decimal(1)
        for k in range(40):
            s += term_s
            c += term_c
            term_s *= -t * t / ((2 * k + 2) * (2 * k + 3))
            term_c *= -t * t / ((2 * k + 1) * (2 * k + 2))
        return s, c

    xs = [0.0, 1e-9, 0.125, 0.25, np.nextafter(0.25, 1), 0.3, 0.49999, 0.5]
    xs += list(np.random.default_rng(3).uniform(0, 0.5, 400))
    sp, cp = (ctypes.c_float * 2)(), (ctypes.c_float * 2)()
    worst = 0.0
    for x in xs:
        lib.afmib_test_sincospi(float(x), sp, cp)
        s_ex, c_ex = exact(float(x))
        got_s = Decimal(float(sp[0])) + Decimal(float(sp[1]))
        got_c = Decimal(float(cp[0])) + Decimal(float(cp[1]))
        scale = max(abs(s_ex), abs(c_ex))
        worst = max(worst, float(abs(got_s - s_ex) / scale), float(abs(got_c - c_ex) / scale))
    assert worst < 2.0 ** -44, worst
