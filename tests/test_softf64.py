"""Integer-pipe binary64 add / sub / mul / reciprocal (csrc/softf64.cuh), built for the
host and compared bit for bit with the host's IEEE 754 arithmetic (numpy) on
random operands of every magnitude relation, on rounding ties, cancellations,
zeros, subnormals, overflow and NaN/infinity.  Where the fast path declines
(NaN or infinite operands, subnormal or overflowing results), the kernels
use the hardware instruction; the test checks that it declines exactly
there and nowhere a normal result is expected.  No GPU needed."""

from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "stencil_benchmarks_gb300" / "csrc"
HARNESS = Path(__file__).resolve().parent / "native" / "softf64_harness.cpp"


@pytest.fixture(scope="module")
def sf(tmp_path_factory):
    out = tmp_path_factory.mktemp("softf64") / "libsoftf64.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{CSRC}",
                    str(HARNESS), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    up = ctypes.POINTER(ctypes.c_uint64)
    lib.sf_binop.argtypes = [ctypes.c_int, up, up, up, ctypes.POINTER(ctypes.c_ubyte), ctypes.c_long]
    lib.sf_set_rcp_perturb.argtypes = [ctypes.c_int]
    return lib


def run(sf, op, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.empty(len(a), dtype=np.uint64)
    taken = np.empty(len(a), dtype=np.uint8)
    up = ctypes.POINTER(ctypes.c_uint64)
    sf.sf_binop(op, a.view(np.uint64).ctypes.data_as(up), b.view(np.uint64).ctypes.data_as(up),
                out.ctypes.data_as(up), taken.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), len(a))
    return out, taken.astype(bool)


def expected(op, a, b):
    with np.errstate(all="ignore"):
        return {0: np.add, 1: np.subtract, 2: np.multiply}[op](a, b)


def check(sf, op, a, b):
    got, taken = run(sf, op, a, b)
    want = expected(op, a, b)
    wbits = want.view(np.uint64)
    same = got[taken] == wbits[taken]
    assert same.all(), (f"op {op}: {np.count_nonzero(~same)} of {taken.sum()} differ, first "
                        f"{a[taken][~same][:3]} {b[taken][~same][:3]}")
    # declined exactly where a NaN/inf operand or a non-normal result (before rounding) is involved
    special = ~np.isfinite(a) | ~np.isfinite(b)
    tiny = np.abs(want) < 2.0**-1022
    huge = np.abs(want) >= np.finfo(np.float64).max
    declined = special.copy()
    if op == 2:
        zero_operand = ((a == 0) & np.isfinite(b)) | ((b == 0) & np.isfinite(a))
        subnormal = ((np.abs(a) < 2.0**-1022) & (a != 0)) | ((np.abs(b) < 2.0**-1022) & (b != 0))
        declined |= subnormal & ~zero_operand
        tiny &= ~zero_operand
    else:
        tiny &= want != 0
    assert taken[~(declined | tiny | huge)].all(), "fast path declined an ordinary case"
    assert not taken[declined].any(), "fast path took a case it must leave to the hardware"
    return taken


def operands(n, seed, span):
    rng = np.random.Generator(np.random.PCG64(seed))
    e = rng.integers(-span, span + 1, size=(2, n))
    m = rng.uniform(1.0, 2.0, size=(2, n))
    s = rng.choice([-1.0, 1.0], size=(2, n))
    with np.errstate(over="ignore"):
        x = s * m * np.exp2(e.astype(np.float64))
    return x[0], x[1]


@pytest.mark.parametrize("op", [0, 1, 2])
@pytest.mark.parametrize("span", [0, 2, 30, 70, 1100])
def test_random_operands(sf, op, span):
    a, b = operands(200_000, 10 + span + op, span)
    check(sf, op, a, b)


@pytest.mark.parametrize("op", [0, 1, 2])
def test_stencil_like_values(sf, op):
    """U[0,1) and U[-1,1) values as the workloads draw them (all exponents
    down to 2^-53 appear, with equal and nearly equal neighbours)."""
    rng = np.random.Generator(np.random.PCG64(7))
    a = rng.uniform(0.0, 1.0, size=300_000)
    b = np.concatenate([rng.uniform(-1.0, 1.0, size=200_000), a[:100_000] * (1 + 2.0**-52)])
    check(sf, op, a, b)
    check(sf, op, a, -a)


def test_rounding_ties_and_cancellation(sf):
    one = 1.0
    ulp = 2.0**-52
    a = np.array([one, one, one + ulp, one + 2 * ulp, 2.0 - ulp, one, 1.5, 3.0, -one, one + ulp, 2.0**53,
                  2.0**53 + 2, 1.0, 1e16, 0.1, 0.3])
    b = np.array([ulp / 2, ulp / 2 * 3, ulp / 2, ulp / 2, ulp / 2, -one, -1.5 + ulp, -3.0 + 4 * ulp, one - ulp,
                  -one, 1.0, 1.0, -ulp / 4, 1.0, 0.2, -0.1])
    for op in (0, 1):
        check(sf, op, a, b)
        check(sf, op, b, a)
    # products that round at an exact tie
    x = 1.0 + np.arange(1, 2000) * 2.0**-27
    check(sf, 2, x, x)
    check(sf, 2, x, 1.0 + 2.0**-26 - x * 2.0**-28)


def test_zeros_subnormals_infinities_nans(sf):
    sub = np.array([5e-324, 2.2250738585072009e-308, -1e-310, 1e-320])
    vals = np.concatenate([np.array([0.0, -0.0, 1.0, -2.5, np.inf, -np.inf, np.nan, 1e308, -1e308, 2.0**-1022,
                                     2.0**-1021, 1.7976931348623157e308, 2.0**1023]), sub])
    a, b = np.meshgrid(vals, vals)
    for op in (0, 1, 2):
        check(sf, op, a.ravel(), b.ravel())
    # results that overflow (declined) and that round up to exactly infinity (taken)
    m = np.finfo(np.float64).max
    check(sf, 0, np.array([m, m, m]), np.array([m, 2.0**970, 2.0**969]))
    check(sf, 2, np.array([m, 2.0**1000, 1.5 * 2.0**1023]), np.array([1.0 + 2.0**-52, 2.0**24, 1.0 + 2.0**-30]))
    # products near the bottom of the normal range
    check(sf, 2, np.array([2.0**-511, 2.0**-512, 1.5 * 2.0**-511, 2.0**-1000]),
          np.array([2.0**-511, 2.0**-511, 1.5 * 2.0**-512, 2.0**-22]))


# ---------------------------------------------------------------------------
# reciprocal
# ---------------------------------------------------------------------------


def check_rcp(sf, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    got, taken = run(sf, 3, a, a)
    with np.errstate(all="ignore"):
        want = (1.0 / a).view(np.uint64)
    same = got[taken] == want[taken]
    assert same.all(), f"rcp: {np.count_nonzero(~same)} of {taken.sum()} differ, first {a[taken][~same][:3]}"
    # declined exactly for zeros, subnormals, inf/NaN and |a| >= 2^1022
    absa = np.abs(a)
    declined = ~np.isfinite(a) | (absa < 2.0**-1022) | (absa >= 2.0**1022)
    assert taken[~declined].all(), "rcp declined an ordinary operand"
    assert not taken[declined].any(), "rcp took an operand it must leave to the hardware"


@pytest.mark.parametrize("perturb", [0, -8, -3, -1, 1, 3, 8])
def test_rcp_random_significands(sf, perturb):
    """Every significand region, with the float seed moved by up to 8 ulps
    either way (the device seeds with rcp.approx, within about 1 ulp): the
    two Newton steps and the remainder correction absorb it."""
    sf.sf_set_rcp_perturb(perturb)
    try:
        rng = np.random.Generator(np.random.PCG64(100 + perturb))
        n = 400_000
        m = 1.0 + rng.integers(1, 2**52, size=n, dtype=np.int64).astype(np.float64) * 2.0**-52
        e = rng.integers(-1000, 1000, size=n)
        s = rng.choice([-1.0, 1.0], size=n)
        check_rcp(sf, s * m * np.exp2(e.astype(np.float64)))
    finally:
        sf.sf_set_rcp_perturb(0)


@pytest.mark.parametrize("perturb", [0, -8, 8])
def test_rcp_edge_significands(sf, perturb):
    """Significands at the ends of [1, 2), next to powers of two, halves and
    thirds, and those whose seeds sit on float boundaries (the top 24 bits
    all ones or 2^23), where the quotient's last bits are closest to a
    rounding boundary."""
    sf.sf_set_rcp_perturb(perturb)
    try:
        k = np.arange(0, 4096, dtype=np.int64)
        frac = np.concatenate([
            1 + k, 2**52 - 1 - k, 2**51 + k - 2048, (2**52 // 3) + k - 2048, (2 * 2**52 // 3) + k - 2048,
            ((2**24 - 1) << 28) + k, ((2**24 - 1) << 28) - 1 - k, (1 << 28) + k - 2048,
        ])
        frac = frac[(frac > 0) & (frac < 2**52)]
        a = (np.uint64(1023) << np.uint64(52) | frac.astype(np.uint64)).view(np.float64)
        check_rcp(sf, np.concatenate([a, -a, a * 2.0**700, a * 2.0**-700]))
    finally:
        sf.sf_set_rcp_perturb(0)


def test_rcp_stencil_like_values(sf):
    """The denominators the vertical solve takes: U[0.1, 3) as its bcol
    differences draw them, and powers of two."""
    rng = np.random.Generator(np.random.PCG64(11))
    check_rcp(sf, rng.uniform(0.1, 3.0, size=300_000))
    check_rcp(sf, np.exp2(np.arange(-1022, 1024, dtype=np.float64)))


def test_rcp_specials(sf):
    vals = np.array([0.0, -0.0, 5e-324, -1e-310, 2.0**-1022, -2.0**-1022, 2.0**-1021, np.inf, -np.inf, np.nan,
                     2.0**1020, 1.9 * 2.0**1020, 2.0**1021, 1.5 * 2.0**1021, 2.0**1022, 1.5 * 2.0**1022, 2.0**1023,
                     np.finfo(np.float64).max])
    check_rcp(sf, vals)
