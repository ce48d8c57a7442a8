"""Float-pair arithmetic (csrc/f32x2.cuh) built for the host and checked
against exact rational arithmetic: conversions keep 48+ bits, add/sub/mul/
div/rcp stay within a few 2^-48 (absolute of the operands for add/sub),
comparisons are exact on the converted values.  No GPU needed."""

from __future__ import annotations

import ctypes
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "stencil_benchmarks_gb300" / "csrc"
HARNESS = Path(__file__).resolve().parent / "native" / "f32x2_harness.cpp"


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    out = tmp_path_factory.mktemp("f32x2") / "libf32x2.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{CSRC}",
                    str(HARNESS), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    dp, fp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)
    lib.fx_split.argtypes = [dp, fp, fp, ctypes.c_long]
    lib.fx_join.argtypes = [fp, fp, dp, ctypes.c_long]
    lib.fx_binop.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_long]
    return lib


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def split(fx, x):
    hi, lo = np.empty(len(x), np.float32), np.empty(len(x), np.float32)
    fx.fx_split(_p(x, ctypes.c_double), _p(hi, ctypes.c_float), _p(lo, ctypes.c_float), len(x))
    return hi, lo


def binop(fx, op, a, b=None):
    b = a if b is None else b
    out = np.empty(len(a))
    fx.fx_binop(op, _p(a, ctypes.c_double), _p(b, ctypes.c_double), _p(out, ctypes.c_double), len(a))
    return out


def samples(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    mags = rng.uniform(-30, 30, size=n)
    x = rng.uniform(0.5, 1.0, size=n) * np.exp2(np.round(mags)) * rng.choice([-1.0, 1.0], size=n)
    edge = np.array([1.0, -1.0, 0.1, 1 / 3, 2.0**-100, 1.0 + 2.0**-52, 1.0 - 2.0**-53, 0.15, 3.0,
                     np.nextafter(1.0, 2.0), np.nextafter(2.0, 0.0), 1e30, -1e-30])
    return np.concatenate([edge, x])


def test_split_keeps_48_bits_and_is_normalised(fx):
    x = samples(4000, 1)
    hi, lo = split(fx, x)
    for xv, h, l in zip(x, hi, lo):
        err = abs(Fraction(float(h)) + Fraction(float(l)) - Fraction(float(xv)))
        assert err <= Fraction(abs(float(xv))) * Fraction(1, 2**49), (xv, h, l)
        if h != 0:
            ulp = np.spacing(np.float32(abs(h)))
            assert abs(float(l)) <= float(ulp) / 2, (xv, h, l)


def test_split_special_values(fx):
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e300, 1e-300, 2.0**-130])
    hi, lo = split(fx, x)
    assert hi[0] == 0 and lo[0] == 0 and np.signbit(hi[1])
    assert hi[2] == np.inf and hi[3] == -np.inf and np.isnan(hi[4])
    assert hi[5] == np.inf  # beyond the float32 range
    assert hi[6] == 0.0 or abs(hi[6]) < 1e-38
    assert hi[7] == np.float32(2.0**-130)  # float32 subnormal, float32 precision


def test_round_trip_within_one_ulp_of_48_bits(fx):
    x = samples(4000, 2)
    back = binop(fx, 7, binop(fx, 7, x))  # neg(neg(x)) through split and join
    rel = np.abs(back - x) / np.abs(x)
    assert rel.max() <= 2.0**-48


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_binary_ops_error_bounds(fx, op):
    a, b = samples(3000, 3 + op), samples(3000, 13 + op)[::-1].copy()
    got = binop(fx, op, a, b)
    for av, bv, g in zip(a, b, got):
        A, B = Fraction(float(av)), Fraction(float(bv))
        exact = [A + B, A - B, A * B, A / B][op]
        err = abs(Fraction(float(g)) - exact)
        if exact != 0 and abs(exact) < Fraction(1, 2**100):
            continue  # below the full-precision range (the low word is subnormal)
        if op in (0, 1):
            assert err <= (abs(A) + abs(B)) * Fraction(1, 2**45), (op, av, bv, g)
        else:
            assert err <= abs(exact) * Fraction(1, 2**45), (op, av, bv, g)


def test_reciprocal_and_scale(fx):
    a = samples(3000, 7)
    r = binop(fx, 4, a)
    assert np.all(np.abs(r * a - 1.0) <= 2.0**-45)
    s = binop(fx, 6, a)
    assert np.all(np.abs(s - 4 * a) <= np.abs(4 * a) * 2.0**-48)


def test_compare_is_exact_on_split_values(fx):
    a = samples(2000, 8)
    b = a.copy()
    b[::3] = np.nextafter(b[::3], np.inf)  # differs below 48 bits: may compare equal
    b[1::3] = b[1::3] * (1 + 2.0**-40)
    c = binop(fx, 5, a, b)
    ha, la = split(fx, a)
    hb, lb = split(fx, b)
    for q in range(len(a)):
        va = Fraction(float(ha[q])) + Fraction(float(la[q]))
        vb = Fraction(float(hb[q])) + Fraction(float(lb[q]))
        want = (va > vb) - (va < vb)
        assert c[q] == want
