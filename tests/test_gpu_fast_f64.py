"""The fast float64 forms on the GPU against the float64 oracle, within the
stated tolerances:

    hdiff: max |got - oracle| <= 1e-12 * max |oracle|
    vadv:  max |got - oracle| <= 1e-10 * max |oracle| on well-conditioned
           domains; on ill-conditioned ones the float-pair solve is held to
           2^10 times float64's own error instead (its error grows with the
           column's conditioning, so 1e-10 is not a property it has there)

(relative to the field's magnitude).  Float-pair compute ("float32x2")
carries about 48 significant bits, so isolated results close to zero have
large pointwise relative errors while their absolute error stays a few 2^-48
of the operands.  Fixed-point hdiff ("fixed64") sums exactly in 64-bit
integers on a per-strip scale and rounds once through a float64 FMA: its
errors are at float64 rounding level, which the tests check as well.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, kernels
from stencil_benchmarks_gb300.batching import Batch, HdiffDomain, VadvDomain
from tests.conftest import golden_cases, load_golden
from tests.gpu_helpers import (
    VADV_ARGS,
    VADV_DISTS,
    download_like,
    host_field,
    interior,
    rng_fields,
    to_device,
)

pytestmark = pytest.mark.gpu

HDIFF_TOL = 1e-12
VADV_TOL = 1e-10


def _check(got, want, tol, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert got.shape == want.shape
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    err = float(np.max(np.abs(got - want))) if want.size else 0.0
    assert np.all(np.isfinite(got)), f"{what}: non-finite results"
    assert err <= tol * max(scale, 1e-300), f"{what}: max abs error {err:.3e} > {tol:g} * {scale:.3e}"
    return err / max(scale, 1e-300)


def _hdiff(domain, halo, tune=None, seed=0, layout=(2, 1, 0), alignment=0):
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(seed, shape, ("inp", "coeff", "out"), {})
    hosts = {n: host_field(v, "float64", layout, alignment, halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute="float32x2", tune=tune)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    return got, want


@pytest.mark.parametrize("variant", [_native.HDIFF_TILE, _native.HDIFF_JSCAN])
@pytest.mark.parametrize("domain,halo,layout", [((150, 97, 6), (2, 2, 0), (2, 1, 0)),
                                                ((33, 130, 2), (2, 4, 2), (0, 1, 2)),
                                                ((1, 1, 1), (2, 2, 0), (2, 1, 0))])
def test_hdiff_pair(variant, domain, halo, layout, lib):
    got, want = _hdiff(domain, halo, tune=_native.tune(variant=variant), seed=21, layout=layout)
    _check(got, want, HDIFF_TOL, f"hdiff pair variant {variant} {domain}")


@pytest.mark.parametrize("domain,halo", [((150, 97, 6), (2, 2, 0)), ((77, 45, 3), (3, 3, 1))])
def test_hdiff_pair_vscan(domain, halo, lib):
    """Vector strips compute the same pair arithmetic per point as JSCAN: same bits."""
    got, want = _hdiff(domain, halo, tune=_native.tune(variant=_native.HDIFF_VSCAN), seed=23, alignment=64)
    _check(got, want, HDIFF_TOL, f"hdiff pair vscan {domain}")
    ref, _ = _hdiff(domain, halo, tune=_native.tune(variant=_native.HDIFF_JSCAN), seed=23, alignment=64)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("domain,halo", [((150, 97, 6), (2, 2, 0)), ((77, 45, 3), (3, 3, 1))])
def test_hdiff_pair_tma(domain, halo, lib):
    """The TMA-staged tile computes the same pair arithmetic as TILE: same bits."""
    got, want = _hdiff(domain, halo, tune=_native.tune(variant=_native.HDIFF_TMA), seed=22, alignment=64)
    _check(got, want, HDIFF_TOL, f"hdiff pair tma {domain}")
    tile, _ = _hdiff(domain, halo, tune=_native.tune(variant=_native.HDIFF_TILE, block_x=64, block_y=4,
                                                     tile_y=16, k_per_cta=8), seed=22, alignment=64)
    assert np.array_equal(got.view(np.uint64), tile.view(np.uint64))


def _vadv(domain, halo, tune=None, seed=0, shift=(1, 0), use_scratch=False):
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(seed, shape, VADV_ARGS, VADV_DISTS)
    hosts = {n: host_field(v, "float64", (2, 1, 0), 0, halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    scratch = {}
    if use_scratch:  # pair factors fit in float64-sized scratch elements
        for n in ("ccol", "dcol"):
            scratch[n] = to_device(host_field(np.zeros(shape), "float64", (2, 1, 0), 0, halo), "float64", halo)
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], shift,
                 ccol=scratch.get("ccol"), dcol=scratch.get("dcol"), compute="float32x2", tune=tune)
    got = interior(download_like(dev["utensstage"], hosts["utensstage"]), domain, halo)
    f = {n: np.array(h) for n, h in hosts.items()}
    want = ora._vadv_component(f["ustage"], f["upos"], f["utens"], f["utensstage"], f["wcon"], domain, halo,
                               shift[0], shift[1])
    return got, want


@pytest.mark.parametrize("variant,bx,by,depth", [(0, 0, 0, 0), (1, 32, 1, 4), (1, 64, 1, 8), (1, 32, 2, 2),
                                                 (2, 32, 1, 4), (2, 128, 2, 8), (3, 32, 1, 4), (3, 64, 1, 2),
                                                 (3, 32, 1, 1), (4, 32, 1, 4), (4, 64, 1, 2)])
def test_vadv_pair_variants(variant, bx, by, depth, lib):
    t = _native.tune(variant=variant, block_x=bx, block_y=by, unroll=depth)
    for nk in (2, 3, 9, 40):
        got, want = _vadv((97, 19, nk), (1, 1, 0), tune=t, seed=30 + nk, use_scratch=(variant in (2, 3, 4)))
        _check(got, want, VADV_TOL, f"vadv pair variant {variant} {bx}x{by} depth {depth} nk {nk}")


@pytest.mark.parametrize("shift", [(1, 0), (0, 1), (0, 0)])
def test_vadv_pair_shifts(shift, lib):
    """With wcon shift (0, 0) these random columns are ill-conditioned (results
    up to ~4e4): float64 itself is then ~7e-12 of the scale away from the
    exact solution, and the pair's error grows by the same conditioning.  The
    bound is 1e-10 of the scale or 2^10 times float64's own error (measured
    against the oracle in extended precision), whichever is larger."""
    domain, halo = (45, 20, 17), (1, 1, 1)
    got, want = _vadv(domain, halo, seed=41, shift=shift)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(41, shape, VADV_ARGS, VADV_DISTS)
    ext = ora._vadv_component(*[vals[n].astype(np.longdouble) for n in VADV_ARGS], domain, halo, *shift)
    fp64_err = float(np.max(np.abs(np.asarray(want, np.longdouble) - ext)))
    scale = float(np.max(np.abs(want)))
    err = float(np.max(np.abs(np.asarray(got, np.float64) - want)))
    assert err <= max(VADV_TOL * scale, 2.0**10 * fp64_err), (shift, err, scale, fp64_err)


@pytest.mark.parametrize("name", [n for n, m in golden_cases().items()
                                  if not n.startswith("_") and m["kind"] in ("hdiff", "vadv")
                                  and m["dtype"] == "float64"])
def test_golden_pair(name, lib):
    """The reference's own golden vectors, computed in float pairs."""
    meta = golden_cases()[name]
    data = load_golden(name)
    domain, halo = tuple(meta["domain"]), tuple(meta["halo"])
    hosts = {n: host_field(data[f"in_{n}"], "float64", halo=halo) for n in meta["args"]}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    if meta["kind"] == "hdiff":
        kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute="float32x2")
        pairs, tol = {"out": "out"}, HDIFF_TOL
    else:
        kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], (1, 0),
                     compute="float32x2")
        pairs, tol = {"utensstage": "utensstage"}, VADV_TOL
        if meta["params"].get("all_components"):
            kernels.vadv(dev["vstage"], dev["vpos"], dev["vtens"], dev["vtensstage"], dev["wcon"], (0, 1),
                         compute="float32x2")
            kernels.vadv(dev["wstage"], dev["wpos"], dev["wtens"], dev["wtensstage"], dev["wcon"], (0, 0),
                         compute="float32x2")
            pairs.update(vtensstage="vtensstage", wtensstage="wtensstage")
    _native.synchronize()
    shifts = {"utensstage": (1, 0), "vtensstage": (0, 1), "wtensstage": (0, 0)}
    for expected, field in pairs.items():
        got = interior(download_like(dev[field], hosts[field]), domain, halo)
        want = data[f"expected_{expected}"]
        if meta["kind"] == "hdiff":
            _check(got, want, tol, f"{name}:{expected}")
            continue
        c = expected[0]  # u, v or w
        ins = [data[f"in_{c}{n}"].astype(np.longdouble) for n in ("stage", "pos", "tens", "tensstage")]
        ext = ora._vadv_component(*ins, data["in_wcon"].astype(np.longdouble), domain, halo, *shifts[expected])
        fp64_err = float(np.max(np.abs(np.asarray(want, np.longdouble) - ext)))
        err = float(np.max(np.abs(np.asarray(got, np.float64) - want)))
        scale = float(np.max(np.abs(want)))
        assert err <= max(tol * scale, 2.0**10 * fp64_err), (name, expected, err, scale, fp64_err)


def test_batch_pair(lib):
    """Uneven hdiff and vadv domains in one batch launch, float pairs."""
    rng = np.random.Generator(np.random.PCG64(51))
    batch = Batch("float64", "float32x2", max_domains=8, max_nk=48)
    doms, checks = [], []
    for q in range(8):
        ni, nj, nk = (int(v) for v in (rng.integers(20, 90), rng.integers(10, 60), rng.integers(2, 48)))
        if q % 2 == 0:
            halo = (2, 2, 0)
            shape = (ni + 4, nj + 4, nk)
            vals = rng_fields(60 + q, shape, ("inp", "coeff", "out"), {})
            hosts = {n: host_field(v, "float64", halo=halo) for n, v in vals.items()}
            dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
            doms.append(HdiffDomain(dev["inp"], dev["coeff"], dev["out"]))
            want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), (ni, nj, nk), halo)
            checks.append((dev["out"], hosts["out"], (ni, nj, nk), halo, want, HDIFF_TOL))
        else:
            halo = (1, 1, 0)
            shape = (ni + 2, nj + 2, nk)
            vals = rng_fields(60 + q, shape, VADV_ARGS + ("out",), VADV_DISTS)
            hosts = {n: host_field(v, "float64", halo=halo) for n, v in vals.items()}
            dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
            doms.append(VadvDomain(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"],
                                   out=dev["out"]))
            f = {n: np.array(h) for n, h in hosts.items()}
            want = ora._vadv_component(f["ustage"], f["upos"], f["utens"], f["utensstage"], f["wcon"],
                                       (ni, nj, nk), halo, 1, 0)
            checks.append((dev["out"], hosts["out"], (ni, nj, nk), halo, want, VADV_TOL))
    batch.set(doms)
    batch.launch()
    _native.synchronize()
    for q, (field, host, domain, halo, want, tol) in enumerate(checks):
        got = interior(download_like(field, host), domain, halo)
        _check(got, want, tol, f"batch domain {q}")


# ---------------------------------------------------------------------------
# fixed-point hdiff
# ---------------------------------------------------------------------------



def _hdiff_values(domain, halo, inp, coeff, tune=None, compute="fixed64"):
    hosts = {"inp": host_field(inp, "float64", halo=halo), "coeff": host_field(coeff, "float64", halo=halo),
             "out": host_field(np.zeros_like(inp), "float64", halo=halo)}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute=compute, tune=tune)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    return got, want


@pytest.mark.parametrize("domain,halo,layout", [((150, 97, 6), (2, 2, 0), (2, 1, 0)),
                                                ((33, 130, 2), (2, 4, 2), (0, 1, 2)),
                                                ((1, 1, 1), (2, 2, 0), (2, 1, 0)),
                                                ((512, 64, 3), (2, 2, 0), (2, 1, 0))])
@pytest.mark.parametrize("tune", [None, dict(block_y=2, tile_y=8, unroll=1), dict(block_y=8, tile_y=64, unroll=8)])
def test_hdiff_fixed(domain, halo, layout, tune, lib):
    t = _native.tune(variant=_native.HDIFF_JSCAN, **tune) if tune else None
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(23, shape, ("inp", "coeff", "out"), {})
    hosts = {n: host_field(v, "float64", layout, 0, halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute="fixed64", tune=t)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    rel = _check(got, want, HDIFF_TOL, f"hdiff fixed {domain} {tune}")
    assert rel <= 2.0**-50, rel  # float64 rounding level


def test_hdiff_fixed_wide_magnitudes(lib):
    """Inputs spanning 8 decades lose bits under the strip's unit: the error
    stays at float64 rounding level of the field scale.  Strips spanning more
    than 2^40 (here 20 decades) run the float64 strip: bit-identical."""
    domain, halo = (96, 70, 4), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(24))
    sign = rng.choice([-1.0, 1.0], size=shape)
    coeff = rng.uniform(0, 1, size=shape)
    got, want = _hdiff_values(domain, halo, 10.0 ** rng.uniform(-8, 0, size=shape) * sign, coeff)
    rel = _check(got, want, HDIFF_TOL, "hdiff fixed 8 decades")
    assert rel <= 2.0**-50, rel
    got, want = _hdiff_values(domain, halo, 10.0 ** rng.uniform(-20, 0, size=shape) * sign, coeff)
    assert np.array_equal(got.view(np.uint64), np.asarray(want).view(np.uint64))


def test_hdiff_fixed_fallback_strips(lib):
    """Strips holding nan/inf, huge (>= 2^1017) or only tiny (< 2^-500)
    values, or only zeros, run the float64 strip: bit-identical to the
    oracle there; every other strip stays within the tolerance."""
    domain, halo = (200, 120, 3), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(25))
    inp = rng.uniform(0, 1, size=shape)
    coeff = rng.uniform(0, 1, size=shape)
    inp[10, 5, 0] = np.nan
    inp[40, 60, 1] = np.inf
    inp[100:130, 0:40, 2] = rng.uniform(-1, 1, size=(30, 40)) * 2.0**1020
    inp[0:60, 80:124, 0] = rng.uniform(-1, 1, size=(60, 44)) * 2.0**-700
    inp[150:204, 50:124, 1] = 0.0
    got, want = _hdiff_values(domain, halo, inp, coeff)
    nan_got, nan_want = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_got, nan_want)
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    g, w = got[fin], want[fin]
    big = np.abs(w) > 1e300
    assert np.all(np.abs(g[big] - w[big]) <= 1e-12 * np.abs(w[big]).max())
    small = ~big
    assert np.max(np.abs(g[small] - w[small])) <= 1e-12 * np.abs(w[small]).max()


def test_golden_fixed(lib):
    for name, meta in golden_cases().items():
        if name.startswith("_") or meta["kind"] != "hdiff" or meta["dtype"] != "float64":
            continue
        data = load_golden(name)
        domain, halo = tuple(meta["domain"]), tuple(meta["halo"])
        got, _ = _hdiff_values(domain, halo, data["in_inp"], data["in_coeff"])
        _check(got, data["expected_out"], HDIFF_TOL, f"{name} fixed")


@pytest.mark.parametrize("storage,compute", [("float64", "fixed64")])
def test_batch_mixed_forms(storage, compute, lib):
    """Batches of the mixed fast float64 form: fixed-point hdiff with
    float-pair vadv on float64 storage."""
    rng = np.random.Generator(np.random.PCG64(52))
    batch = Batch(storage, compute, max_domains=6, max_nk=48)
    doms, checks = [], []
    for q in range(6):
        ni, nj, nk = (int(v) for v in (rng.integers(20, 90), rng.integers(10, 60), rng.integers(2, 48)))
        if q % 2 == 0:
            halo = (2, 2, 0)
            vals = rng_fields(80 + q, (ni + 4, nj + 4, nk), ("inp", "coeff", "out"), {})
            hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
            dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
            doms.append(HdiffDomain(dev["inp"], dev["coeff"], dev["out"]))
            # float32 hdiff is plain float32: bit-identical to the oracle in float32
            want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), (ni, nj, nk), halo)
            tol = HDIFF_TOL if storage == "float64" else 0.0
            checks.append((dev["out"], hosts["out"], (ni, nj, nk), halo, want, tol))
        else:
            halo = (1, 1, 0)
            vals = rng_fields(80 + q, (ni + 2, nj + 2, nk), VADV_ARGS + ("out",), VADV_DISTS)
            hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
            dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
            doms.append(VadvDomain(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"],
                                   out=dev["out"]))
            f = {n: np.array(h, np.float64) for n, h in hosts.items()}
            want = ora._vadv_component(f["ustage"], f["upos"], f["utens"], f["utensstage"], f["wcon"],
                                       (ni, nj, nk), halo, 1, 0)
            checks.append((dev["out"], hosts["out"], (ni, nj, nk), halo, want,
                           VADV_TOL if storage == "float64" else 1e-5))
    batch.set(doms)
    batch.launch()
    _native.synchronize()
    for q, (field, host, domain, halo, want, tol) in enumerate(checks):
        got = interior(download_like(field, host), domain, halo)
        _check(got, want, tol, f"batch {storage}/{compute} domain {q}")
