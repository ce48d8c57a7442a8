"""float64 kernels with part of their operations in integer arithmetic
(csrc/softf64.cuh): every placement preset of the hdiff TMA tile and of the
vadv SLAB form must stay bit-identical to the oracle, on ordinary workload
values and on values that take the integer path's fallbacks (zeros,
subnormal operands and results, overflow to infinity, NaN); and the device
build of the integer operations themselves (the reciprocal seeds with the
device's approximate instruction) against IEEE arithmetic."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, kernels
from tests.gpu_helpers import (
    VADV_ARGS,
    VADV_DISTS,
    bits_equal,
    download_like,
    host_field,
    interior,
    mismatch_report,
    rng_fields,
    to_device,
)

pytestmark = pytest.mark.gpu

HDIFF_PRESETS = range(1, 9)
VADV_PRESETS = range(1, 16)


def _specials(rng, shape, scale):
    """Workload values with a sprinkling of zeros, subnormals, huge values and NaN."""
    v = rng.uniform(-scale, scale, size=shape)
    pick = rng.random(size=shape)
    v[pick < 0.02] = 0.0
    v[(pick >= 0.02) & (pick < 0.03)] = 3e-310
    v[(pick >= 0.03) & (pick < 0.035)] = -2.2250738585072014e-308
    v[(pick >= 0.035) & (pick < 0.04)] = 1.5e308
    v[(pick >= 0.04) & (pick < 0.041)] = np.nan
    return v


@pytest.mark.parametrize("preset", HDIFF_PRESETS)
@pytest.mark.parametrize("special", [False, True])
def test_hdiff_tma_placements(preset, special, lib):
    domain, halo = (130, 70, 6), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(100 + preset))
    vals = {n: (_specials(rng, shape, 1.0) if special else rng.uniform(0.0, 1.0, size=shape))
            for n in ("inp", "coeff", "out")}
    hosts = {n: host_field(v, alignment=64, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], tune=_native.tune(flags=preset << 4))
    _native.synchronize()
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    with np.errstate(all="ignore"):
        want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    assert bits_equal(got, want), f"preset {preset}: " + mismatch_report(got, want)


@pytest.mark.parametrize("preset", VADV_PRESETS)
@pytest.mark.parametrize("per_sm", [0, 24])
@pytest.mark.parametrize("nk", [2, 3, 40])
def test_vadv_slab_placements(preset, per_sm, nk, lib):
    domain, halo = (97, 19, nk), (1, 1, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(200 + preset + nk, shape, VADV_ARGS, VADV_DISTS)
    hosts = {n: host_field(v, halo=halo) for n, v in vals.items()}
    for n in ("out", "ccol", "dcol"):
        hosts[n] = host_field(np.zeros(shape), halo=halo)
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    tune = _native.tune(variant=_native.VADV_SLAB, block_x=32, unroll=1, k_per_cta=per_sm, flags=preset << 4)
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], out=dev["out"],
                 ccol=dev["ccol"], dcol=dev["dcol"], tune=tune)
    _native.synchronize()
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora._vadv_component(*(np.array(hosts[n]) for n in VADV_ARGS), domain, halo, 1, 0)
    assert bits_equal(got, want), f"preset {preset}, {per_sm} blocks/SM, nk {nk}: " + mismatch_report(got, want)


@pytest.mark.parametrize("preset", [2, 5, 9, 10, 11, 15])
def test_vadv_slab_placements_with_specials(preset, lib):
    domain, halo = (64, 12, 30), (1, 1, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(300 + preset))
    vals = {n: _specials(rng, shape, 1.0 if n != "wcon" else 0.5) for n in VADV_ARGS}
    hosts = {n: host_field(v, halo=halo) for n, v in vals.items()}
    for n in ("out", "ccol", "dcol"):
        hosts[n] = host_field(np.zeros(shape), halo=halo)
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    tune = _native.tune(variant=_native.VADV_SLAB, block_x=32, unroll=1, flags=preset << 4)
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], out=dev["out"],
                 ccol=dev["ccol"], dcol=dev["dcol"], tune=tune)
    _native.synchronize()
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    with np.errstate(all="ignore"):
        want = ora._vadv_component(*(np.array(hosts[n]) for n in VADV_ARGS), domain, halo, 1, 0)
    assert bits_equal(got, want), f"preset {preset}: " + mismatch_report(got, want)


def test_placement_out_of_range_is_rejected(lib):
    domain, halo = (16, 8, 4), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    hosts = {n: host_field(np.zeros(shape), alignment=64, halo=halo) for n in ("inp", "coeff", "out")}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    with pytest.raises(_native.SbError, match="placement"):
        kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], tune=_native.tune(flags=12 << 4))


def test_integer_arithmetic_rates(lib):
    """The probes of the integer binary64 add and multiply and of the two
    leading-zero counts run and report rates."""
    for kind in (8, 9, 10, 11, 14, 15, 16, 17, 18, 19, 20):
        assert kernels.arith_rate(kind) > 1e9


def _soft_on_device(op, a, b):
    """sb_debug_soft_f64 on the device, element-wise."""
    import ctypes

    from stencil_benchmarks_gb300.device import DeviceBuffer, copy_to_device, copy_to_host

    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    da, db, do = (DeviceBuffer(a.nbytes) for _ in range(3))
    copy_to_device(da.ptr, a)
    copy_to_device(db.ptr, b)
    _native.call("sb_debug_soft_f64", op, ctypes.c_void_p(da.ptr), ctypes.c_void_p(db.ptr),
                 ctypes.c_void_p(do.ptr), a.size, None)
    _native.synchronize()
    out = np.empty_like(a)
    copy_to_host(out, do.ptr)
    return out


def _operands(rng, n, span):
    e = rng.integers(-span, span + 1, size=(2, n)).astype(np.float64)
    m = 1.0 + rng.integers(0, 2**52, size=(2, n), dtype=np.int64).astype(np.float64) * 2.0**-52
    s = rng.choice([-1.0, 1.0], size=(2, n))
    with np.errstate(over="ignore"):
        return s[0] * m[0] * np.exp2(e[0]), s[1] * m[1] * np.exp2(e[1])


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_soft_f64_on_device(op, lib):
    """Each integer-arithmetic operation as compiled for sm_103a, on 2 M random
    operands of every magnitude relation plus zeros, subnormals, huge values,
    infinities and NaN: the same bits as numpy (any NaN for a NaN)."""
    rng = np.random.Generator(np.random.PCG64(500 + op))
    a, b = _operands(rng, 2_000_000, 1100 if op == 3 else 60)
    sp = np.array([0.0, -0.0, 5e-324, -3e-310, 2.0**-1022, 1.0, -1.5, 2.0**1021, 1.5 * 2.0**1022,
                   np.finfo(np.float64).max, np.inf, -np.inf, np.nan])
    ga, gb = np.meshgrid(sp, sp)
    # cancellations of every depth: b is a with its lowest t bits redrawn
    # (t = 1..62, so exponent bits too), with the sign that makes op 0 and op 1
    # subtract -- every leading-zero count of the difference, 0 to 63
    near = rng.uniform(-4.0, 4.0, size=200_000)
    t = rng.integers(1, 63, size=near.size).astype(np.uint64)
    low = rng.integers(0, 2**62, size=near.size, dtype=np.int64).astype(np.uint64) & ((np.uint64(1) << t) - np.uint64(1))
    nb = (near.view(np.uint64) & ~((np.uint64(1) << t) - np.uint64(1))) | low
    nb = nb.view(np.float64)
    nb = np.where(np.isfinite(nb), nb, near)
    a = np.concatenate([a, ga.ravel(), rng.uniform(0.1, 3.0, size=100_000), near])
    b = np.concatenate([b, gb.ravel(), rng.uniform(-1.0, 1.0, size=100_000), -nb if op == 0 else nb])
    got = _soft_on_device(op, a, b)
    with np.errstate(all="ignore"):
        want = [a + b, a - b, a * b, 1.0 / a][op]
    nan = np.isnan(want)
    assert (np.isnan(got) == nan).all(), "NaN results differ"
    same = got[~nan].view(np.uint64) == want[~nan].view(np.uint64)
    assert same.all(), f"op {op}: {np.count_nonzero(~same)} differ, first operands {a[~nan][~same][:3]}"


def test_soft_reciprocal_rate(lib):
    """Both reciprocal rate probes run and report a rate: the integer-arithmetic
    reciprocal and the fp64 sequence it replaces (the integer one measured
    faster on GB300, the reason the vadv pivot's reciprocal moved).  No
    ordering is asserted: the probes share the GPU with other work."""
    soft, hard = kernels.arith_rate(12), kernels.arith_rate(13)
    assert soft > 0 and hard > 0
    print(f"reciprocal: integer {soft / 1e9:.1f} G/s, fp64 {hard / 1e9:.1f} G/s")
