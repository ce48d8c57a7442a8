"""float64 kernels with part of their operations in integer arithmetic
(csrc/softf64.cuh): every placement preset of the hdiff TMA tile and of the
vadv SLAB form must stay bit-identical to the oracle, on ordinary workload
values and on values that take the integer path's fallbacks (zeros,
subnormal operands and results, overflow to infinity, NaN)."""

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

PRESETS = range(1, 9)


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


@pytest.mark.parametrize("preset", PRESETS)
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


@pytest.mark.parametrize("preset", PRESETS)
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
    tune = _native.tune(variant=_native.VADV_SLAB, block_x=32, unroll=4, k_per_cta=per_sm, flags=preset << 4)
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], out=dev["out"],
                 ccol=dev["ccol"], dcol=dev["dcol"], tune=tune)
    _native.synchronize()
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora._vadv_component(*(np.array(hosts[n]) for n in VADV_ARGS), domain, halo, 1, 0)
    assert bits_equal(got, want), f"preset {preset}, {per_sm} blocks/SM, nk {nk}: " + mismatch_report(got, want)


@pytest.mark.parametrize("preset", [2, 5])
def test_vadv_slab_placements_with_specials(preset, lib):
    domain, halo = (64, 12, 30), (1, 1, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(300 + preset))
    vals = {n: _specials(rng, shape, 1.0 if n != "wcon" else 0.5) for n in VADV_ARGS}
    hosts = {n: host_field(v, halo=halo) for n, v in vals.items()}
    for n in ("out", "ccol", "dcol"):
        hosts[n] = host_field(np.zeros(shape), halo=halo)
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    tune = _native.tune(variant=_native.VADV_SLAB, block_x=32, unroll=4, flags=preset << 4)
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
    """The probes of the integer binary64 add and multiply run and report rates."""
    for kind in (8, 9, 10, 11):
        assert kernels.arith_rate(kind) > 1e9
