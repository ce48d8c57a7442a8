"""GPU parity: every kernel against the reference's golden vectors and the
CPU oracle, through the C ABI.

fp64 forms must be bit-identical to the reference's numpy verification.  The
reduced-precision forms must be bit-identical to the oracle evaluated on the
same quantised inputs in the same compute type, then rounded once to the
storage type.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, kernels
from tests.conftest import golden_cases, load_golden
from tests.gpu_helpers import (
    VADV_ARGS,
    VADV_DISTS,
    bits_equal,
    compute_view,
    download_like,
    host_field,
    interior,
    mismatch_report,
    rng_fields,
    round_to_storage,
    to_device,
)

pytestmark = pytest.mark.gpu

CASES = {k: v for k, v in golden_cases().items() if not k.startswith("_")}


def _assert_bits(got, want, what):
    assert bits_equal(got, want), f"{what}: " + mismatch_report(got, want)


# ---------------------------------------------------------------------------
# golden vectors captured from the reference
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden(name, lib):
    meta = CASES[name]
    data = load_golden(name)
    storage = meta["dtype"]
    domain, halo = tuple(meta["domain"]), tuple(meta["halo"])
    hosts = {n: host_field(data[f"in_{n}"], storage, halo=halo) for n in meta["args"]}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    kind, params = meta["kind"], meta["params"]
    if kind == "hdiff":
        kernels.hdiff(dev["inp"], dev["coeff"], dev["out"])
        outs = {"out": "out"}
    elif kind == "vadv":
        kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], (1, 0))
        outs = {"utensstage": "utensstage"}
        if params.get("all_components"):
            kernels.vadv(dev["vstage"], dev["vpos"], dev["vtens"], dev["vtensstage"], dev["wcon"], (0, 1))
            kernels.vadv(dev["wstage"], dev["wpos"], dev["wtens"], dev["wtensstage"], dev["wcon"], (0, 0))
            outs.update(vtensstage="vtensstage", wtensstage="wtensstage")
    elif kind == "copy":
        kernels.copy(dev["inp"], dev["out"])
        outs = {"out": "out"}
    elif kind == "laplacian":
        along = (params.get("along_x", True), params.get("along_y", True), params.get("along_z", False))
        kernels.laplacian(dev["inp"], dev["out"], along)
        outs = {"out": "out"}
    elif kind in ("onesided_average", "symmetric_average"):
        kernels.average(dev["inp"], dev["out"], params["axis"], kind == "symmetric_average")
        outs = {"out": "out"}
    else:
        raise AssertionError(kind)
    _native.synchronize()
    for expected_name, field_name in outs.items():
        got = interior(download_like(dev[field_name], hosts[field_name]), domain, halo)
        _assert_bits(got, data[f"expected_{expected_name}"], f"{name}:{expected_name}")


# ---------------------------------------------------------------------------
# horizontal diffusion: shapes, layouts, tunings, precisions
# ---------------------------------------------------------------------------

FORMS = [("float64", "float64"), ("float32", "float32"), ("bfloat16", "float32"), ("float32", "float64")]


def _run_hdiff(domain, halo, storage="float64", compute="float64", layout=(2, 1, 0), alignment=0,
               tune=None, seed=0):
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(seed, shape, ("inp", "coeff", "out"), {})
    hosts = {n: host_field(v, storage, layout, alignment, halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute=compute, tune=tune)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = ora.hdiff(compute_view(hosts["inp"], storage, compute),
                     compute_view(hosts["coeff"], storage, compute), domain, halo)
    return got, round_to_storage(want, storage), hosts


@pytest.mark.parametrize("storage,compute", FORMS)
def test_hdiff_forms(storage, compute, lib):
    got, want, _ = _run_hdiff((150, 97, 6), (2, 2, 0), storage, compute, seed=5)
    _assert_bits(got, want, f"hdiff {storage}/{compute}")


@pytest.mark.parametrize(
    "domain,halo,layout,alignment",
    [
        ((77, 45, 3), (3, 3, 1), (2, 1, 0), 64),
        ((64, 16, 5), (2, 2, 0), (2, 1, 0), 0),
        ((1, 1, 1), (2, 2, 0), (2, 1, 0), 0),
        ((33, 130, 2), (2, 4, 2), (0, 1, 2), 0),
        ((40, 21, 9), (2, 2, 1), (1, 2, 0), 32),
    ],
)
def test_hdiff_shapes_layouts(domain, halo, layout, alignment, lib):
    got, want, _ = _run_hdiff(domain, halo, layout=layout, alignment=alignment, seed=7)
    _assert_bits(got, want, f"hdiff {domain} {halo} {layout}")


@pytest.mark.parametrize("bx,by,ty,kper", [(32, 4, 8, 1), (32, 8, 24, 3), (64, 2, 2, 7), (64, 8, 32, 2),
                                           (128, 2, 4, 1), (128, 4, 16, 5)])
def test_hdiff_tunings(bx, by, ty, kper, lib):
    t = _native.tune(variant=_native.HDIFF_TILE, block_x=bx, block_y=by, tile_y=ty, k_per_cta=kper)
    got, want, _ = _run_hdiff((131, 70, 11), (2, 2, 0), tune=t, seed=9)
    _assert_bits(got, want, f"hdiff tune {bx}x{by} ty{ty} k{kper}")


@pytest.mark.parametrize("storage,compute", [("float64", "float64"), ("float32", "float32"), ("bfloat16", "float32")])
@pytest.mark.parametrize("nw,ty,kper,unroll", [(1, 1, 1, 1), (2, 7, 3, 2), (4, 32, 1, 4), (8, 64, 2, 8), (3, 5, 4, 4)])
def test_hdiff_jscan_tunings(storage, compute, nw, ty, kper, unroll, lib):
    t = _native.tune(variant=_native.HDIFF_JSCAN, block_y=nw, tile_y=ty, k_per_cta=kper, unroll=unroll)
    got, want, _ = _run_hdiff((129, 67, 5), (2, 2, 0), storage, compute, tune=t, seed=10)
    _assert_bits(got, want, f"hdiff jscan {nw} {ty} {kper} {unroll} {storage}")


# TMA staging needs i unit-stride and j/k strides that are multiples of 16
# bytes (alignment=64 pads rows); the halo corner may sit at any element
# offset from a 16-byte boundary (halo 3 and 9 move it).
@pytest.mark.parametrize("storage,compute", FORMS)
@pytest.mark.parametrize("bx,by,ty,kper", [(64, 4, 16, 8), (32, 8, 8, 3), (64, 8, 40, 2), (128, 2, 4, 1),
                                           (128, 4, 12, 5)])
def test_hdiff_tma(storage, compute, bx, by, ty, kper, lib):
    t = _native.tune(variant=_native.HDIFF_TMA, block_x=bx, block_y=by, tile_y=ty, k_per_cta=kper)
    got, want, _ = _run_hdiff((131, 70, 11), (2, 2, 0), storage, compute, alignment=64, tune=t, seed=31)
    _assert_bits(got, want, f"hdiff tma {bx}x{by} ty{ty} k{kper} {storage}/{compute}")


@pytest.mark.parametrize("storage", ["float64", "float32", "bfloat16"])
@pytest.mark.parametrize("domain,halo", [((77, 45, 3), (3, 3, 1)), ((40, 21, 9), (9, 2, 0)),
                                         ((33, 130, 2), (2, 4, 2)), ((1, 1, 1), (2, 2, 0)),
                                         ((64, 16, 5), (5, 2, 3))])
def test_hdiff_tma_corner_offsets(storage, domain, halo, lib):
    compute = "float64" if storage == "float64" else "float32"
    t = _native.tune(variant=_native.HDIFF_TMA)
    got, want, _ = _run_hdiff(domain, halo, storage, compute, alignment=64, tune=t, seed=32)
    _assert_bits(got, want, f"hdiff tma {domain} {halo} {storage}")


@pytest.mark.parametrize("layout,alignment", [((2, 1, 0), 0), ((0, 1, 2), 64)])
def test_hdiff_tma_rejects_unqualified_layouts(layout, alignment, lib):
    """Rows of 135 float32 (540 bytes) or a strided i axis cannot be described
    to the TMA unit: the call fails with SB_ERR_UNSUPPORTED, nothing runs."""
    t = _native.tune(variant=_native.HDIFF_TMA)
    with pytest.raises(_native.SbError) as err:
        _run_hdiff((131, 70, 3), (2, 2, 0), "float32", "float32", layout=layout, alignment=alignment, tune=t)
    assert err.value.code == _native.SB_ERR_UNSUPPORTED
    assert "TMA" in err.value.message


def test_hdiff_tma_full_size_fp32(lib):
    """512x512x80 float32 through the TMA variant, against the oracle."""
    t = _native.tune(variant=_native.HDIFF_TMA)
    got, want, _ = _run_hdiff((512, 512, 80), (2, 2, 0), "float32", "float32", alignment=64, tune=t, seed=33)
    _assert_bits(got, want, "hdiff tma 512x512x80 float32")


VSCAN_WIDTHS = {"float64": (64,), "float32": (64, 128), "bfloat16": (128, 256)}


@pytest.mark.parametrize("storage,compute", FORMS)
@pytest.mark.parametrize("nw,ty,kper,unroll", [(1, 1, 1, 1), (2, 7, 3, 2), (4, 32, 1, 4), (8, 64, 2, 8),
                                               (3, 5, 4, 4)])
def test_hdiff_vscan(storage, compute, nw, ty, kper, unroll, lib):
    """Vector strips (V columns per lane): same bits as the oracle for every
    strip width, including strips that end inside a vector."""
    for width in VSCAN_WIDTHS[storage]:
        t = _native.tune(variant=_native.HDIFF_VSCAN, block_x=width, block_y=nw, tile_y=ty, k_per_cta=kper,
                         unroll=unroll)
        got, want, _ = _run_hdiff((261, 67, 5), (2, 2, 0), storage, compute, alignment=64, tune=t, seed=34)
        _assert_bits(got, want, f"hdiff vscan {width} {nw} {ty} {kper} {unroll} {storage}/{compute}")


@pytest.mark.parametrize("storage", ["float64", "float32", "bfloat16"])
@pytest.mark.parametrize("domain,halo", [((77, 45, 3), (3, 3, 1)), ((40, 21, 9), (9, 2, 0)),
                                         ((33, 130, 2), (2, 4, 2)), ((1, 1, 1), (2, 2, 0)),
                                         ((64, 16, 5), (5, 2, 3)), ((124, 9, 2), (2, 2, 0)),
                                         ((125, 9, 2), (7, 2, 0))])
def test_hdiff_vscan_offsets(storage, domain, halo, lib):
    """Every offset of the interior from a vector boundary (halo 2..9) and
    domains one column either side of a strip boundary."""
    compute = "float64" if storage == "float64" else "float32"
    for width in VSCAN_WIDTHS[storage]:
        t = _native.tune(variant=_native.HDIFF_VSCAN, block_x=width)
        got, want, _ = _run_hdiff(domain, halo, storage, compute, alignment=64, tune=t, seed=35)
        _assert_bits(got, want, f"hdiff vscan {width} {domain} {halo} {storage}")


@pytest.mark.parametrize("layout,alignment", [((2, 1, 0), 0), ((0, 1, 2), 64)])
def test_hdiff_vscan_rejects_unqualified_layouts(layout, alignment, lib):
    t = _native.tune(variant=_native.HDIFF_VSCAN)
    with pytest.raises(_native.SbError) as err:
        _run_hdiff((131, 70, 3), (2, 2, 0), "float32", "float32", layout=layout, alignment=alignment, tune=t)
    assert err.value.code == _native.SB_ERR_UNSUPPORTED
    assert "VSCAN" in err.value.message


def test_hdiff_vscan_rejects_bad_width(lib):
    t = _native.tune(variant=_native.HDIFF_VSCAN, block_x=32)
    with pytest.raises(_native.SbError) as err:
        _run_hdiff((64, 8, 2), (2, 2, 0), "float32", "float32", alignment=64, tune=t)
    assert err.value.code == _native.SB_ERR_INVALID


def test_hdiff_vscan_full_size(lib):
    """512x512x80 float32 and bfloat16 through vector strips, against the oracle
    (unpadded rows of 516 elements: 16-byte vectors for float32, 8-byte for
    bfloat16)."""
    for storage, width in (("float32", 128), ("bfloat16", 128)):
        t = _native.tune(variant=_native.HDIFF_VSCAN, block_x=width)
        got, want, _ = _run_hdiff((512, 512, 80), (2, 2, 0), storage, "float32", tune=t, seed=36)
        _assert_bits(got, want, f"hdiff vscan 512x512x80 {storage}")


def test_hdiff_special_values(lib):
    """Ties, zeros, signed zeros, tiny and huge values, inf and nan."""
    domain, halo = (40, 12, 3), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(3))
    specials = np.array([0.0, -0.0, 1.0, 1.0, 0.5, 1e-300, -1e-300, 5e-324, 1e300, -1e300, np.inf,
                         -np.inf, np.nan, 2.0, 0.125], dtype=np.float64)
    # a third special values, a third coarse values (exact ties), a third random
    pick = rng.integers(0, 3, size=shape)
    inp = np.where(pick == 0, rng.choice(specials, size=shape),
                   np.where(pick == 1, rng.integers(0, 4, size=shape) / 4.0, rng.random(shape)))
    coeff = np.where(rng.random(shape) < 0.2, rng.choice(specials, size=shape), rng.random(shape))
    hosts = {"inp": host_field(inp, halo=halo), "coeff": host_field(coeff, halo=halo),
             "out": host_field(np.zeros(shape), halo=halo)}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"])
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    with np.errstate(all="ignore"):
        want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    _assert_bits(got, want, "hdiff special values")


def test_hdiff_empty_domain_is_noop(lib):
    got, want, _ = _run_hdiff((0, 5, 3), (2, 2, 0))
    assert got.size == 0 and want.size == 0


# ---------------------------------------------------------------------------
# vertical advection
# ---------------------------------------------------------------------------


def _run_vadv(domain, halo, storage="float64", compute="float64", layout=(2, 1, 0), alignment=0,
              tune=None, seed=0, shift=(1, 0), use_scratch=False):
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(seed, shape, VADV_ARGS, VADV_DISTS)
    hosts = {n: host_field(v, storage, layout, alignment, halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    scratch = {}
    if use_scratch:
        for n in ("ccol", "dcol"):
            h = host_field(np.zeros(shape), compute, layout, alignment, halo)
            scratch[n] = to_device(h, compute, halo)
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], shift,
                 ccol=scratch.get("ccol"), dcol=scratch.get("dcol"), compute=compute, tune=tune)
    got = interior(download_like(dev["utensstage"], hosts["utensstage"]), domain, halo)
    fields = {n: compute_view(h, storage, compute) for n, h in hosts.items()}
    comp = ora._vadv_component(fields["ustage"], fields["upos"], fields["utens"], fields["utensstage"],
                               fields["wcon"], domain, halo, shift[0], shift[1])
    return got, round_to_storage(comp, storage)


@pytest.mark.parametrize("storage,compute", FORMS)
def test_vadv_forms(storage, compute, lib):
    got, want = _run_vadv((70, 33, 40), (1, 1, 0), storage, compute, seed=11)
    _assert_bits(got, want, f"vadv {storage}/{compute}")


@pytest.mark.parametrize("shift", [(1, 0), (0, 1), (0, 0)])
def test_vadv_shifts(shift, lib):
    got, want = _run_vadv((45, 20, 17), (1, 1, 1), seed=12, shift=shift)
    _assert_bits(got, want, f"vadv shift {shift}")


@pytest.mark.parametrize("variant,bx,by,depth", [(1, 32, 1, 1), (1, 64, 2, 2), (1, 16, 4, 8), (2, 32, 1, 4),
                                                 (2, 128, 2, 8), (1, 32, 1, 4), (2, 64, 1, 1)])
@pytest.mark.parametrize("storage,compute", [("float64", "float64"), ("float32", "float32")])
def test_vadv_variants(variant, bx, by, depth, storage, compute, lib):
    t = _native.tune(variant=variant, block_x=bx, block_y=by, unroll=depth)
    for nk in (2, 3, 9, 23):  # shorter and longer than the prefetch depth
        got, want = _run_vadv((97, 19, nk), (1, 1, 0), storage, compute, tune=t, seed=13 + nk,
                              use_scratch=(variant == 2))
        _assert_bits(got, want, f"vadv variant {variant} {bx}x{by} depth {depth} nk {nk}")


@pytest.mark.parametrize("variant", [_native.VADV_SLAB, _native.VADV_WSLAB])
@pytest.mark.parametrize("bx,depth,per_sm", [(32, 4, 0), (64, 2, 0), (32, 8, 1), (64, 4, 3)])
@pytest.mark.parametrize("storage,compute", [("float64", "float64"), ("float32", "float32"),
                                             ("bfloat16", "float32")])
def test_vadv_slab(variant, bx, depth, per_sm, storage, compute, lib):
    """Persistent SLAB / WSLAB variants: factors in compact slabs of
    ccol/dcol; few blocks per SM make every thread solve many columns in
    turn; row ends leave warps with 1 or 2 valid lanes (WSLAB)."""
    t = _native.tune(variant=variant, block_x=bx, unroll=depth, k_per_cta=per_sm)
    for domain in ((97, 19, 2), (97, 19, 3), (33, 40, 9), (130, 7, 41)):
        got, want = _run_vadv(domain, (1, 1, 0), storage, compute, tune=t, seed=17 + domain[2], use_scratch=True)
        _assert_bits(got, want, f"vadv slab {variant} {bx} depth {depth} per_sm {per_sm} {domain}")


@pytest.mark.parametrize("per_sm", [0, 1, 28])
@pytest.mark.parametrize("storage,compute", [("float64", "float64"), ("float32", "float32"),
                                             ("bfloat16", "float32")])
def test_vadv_slab_depth_one(per_sm, storage, compute, lib):
    """SLAB with one level of inputs in flight (the float64 default; float
    pairs: tests/test_gpu_fast_f64.py): levels 2 and 3 (no full ring turn)
    and longer columns, one block per SM (every thread many columns) up to
    the default's balanced grid."""
    t = _native.tune(variant=_native.VADV_SLAB, block_x=32, unroll=1, k_per_cta=per_sm)
    for domain in ((97, 19, 2), (97, 19, 3), (33, 40, 9), (130, 7, 41)):
        got, want = _run_vadv(domain, (1, 1, 0), storage, compute, tune=t, seed=23 + domain[2],
                              use_scratch=True)
        _assert_bits(got, want, f"vadv slab depth 1 per_sm {per_sm} {storage}/{compute} {domain}")


@pytest.mark.parametrize("depth", [0, 4, 8, 16])
@pytest.mark.parametrize("storage", ["float32", "bfloat16"])
@pytest.mark.parametrize("staging", [0x400, 0x800], ids=["shared-addr", "generic"])
def test_vadv_tmem(depth, storage, staging, lib):
    """Factors in tensor memory: level counts around the 8-level load window
    and the per-warp column ranges (nk 64 -> 16 warps, 80 -> 12, 128 -> 8,
    256 -> 4 per block), row ends with 1 or 2 valid lanes, many column
    groups per warp; the ring staged through shared addresses and through
    generic pointers."""
    t = _native.tune(variant=_native.VADV_TMEM, unroll=depth, flags=staging)
    for domain in ((97, 19, 2), (97, 19, 3), (33, 40, 9), (130, 7, 41), (64, 5, 64), (40, 6, 80), (35, 3, 128),
                   (34, 2, 137), (33, 2, 256)):
        got, want = _run_vadv(domain, (1, 1, 0), storage, "float32", tune=t, seed=40 + domain[2])
        _assert_bits(got, want, f"vadv tmem depth {depth} {storage} {domain}")


@pytest.mark.parametrize("shift", [(1, 0), (0, 1), (0, 0)])
def test_vadv_tmem_shifts_and_layouts(shift, lib):
    t = _native.tune(variant=_native.VADV_TMEM)
    got, want = _run_vadv((45, 20, 17), (1, 1, 1), "float32", "float32", tune=t, seed=12, shift=shift)
    _assert_bits(got, want, f"vadv tmem shift {shift}")
    got, want = _run_vadv((64, 8, 137), (1, 1, 0), "bfloat16", "float32", alignment=64, tune=t, seed=15,
                          shift=shift)
    _assert_bits(got, want, f"vadv tmem aligned bf16 shift {shift}")


def test_vadv_tmem_full_size(lib):
    """512x512x80 float32: 8192 column groups over 152 blocks of 12 warps."""
    t = _native.tune(variant=_native.VADV_TMEM)
    got, want = _run_vadv((512, 512, 80), (1, 1, 0), "float32", "float32", tune=t, seed=44)
    _assert_bits(got, want, "vadv tmem 512x512x80")


@pytest.mark.parametrize("storage,compute,domain,layout", [
    ("float64", "float64", (40, 6, 9), (2, 1, 0)),    # float64 compute
    ("float32", "float64", (40, 6, 9), (2, 1, 0)),    # float64 compute
    ("float32", "float32", (40, 6, 257), (2, 1, 0)),  # nk > 256
    ("float32", "float32", (40, 6, 9), (0, 1, 2)),    # i not unit-stride
])
def test_vadv_tmem_rejects(storage, compute, domain, layout, lib):
    t = _native.tune(variant=_native.VADV_TMEM)
    with pytest.raises(_native.SbError) as err:
        _run_vadv(domain, (1, 1, 0), storage, compute, layout=layout, tune=t)
    assert err.value.code == _native.SB_ERR_UNSUPPORTED
    assert "TMEM" in err.value.message


@pytest.mark.parametrize(
    "domain,halo,layout,alignment",
    [((5, 4, 2), (1, 1, 0), (2, 1, 0), 0), ((64, 8, 137), (1, 1, 0), (2, 1, 0), 64),
     ((31, 9, 12), (2, 3, 1), (0, 1, 2), 0), ((1, 1, 3), (1, 0, 0), (2, 1, 0), 0)],
)
def test_vadv_shapes_layouts(domain, halo, layout, alignment, lib):
    got, want = _run_vadv(domain, halo, layout=layout, alignment=alignment, seed=14)
    _assert_bits(got, want, f"vadv {domain} {layout}")


def test_vadv_rejects_single_level(lib):
    with pytest.raises(_native.SbError) as err:
        _run_vadv((8, 4, 1), (1, 1, 0))
    assert err.value.code == _native.SB_ERR_INVALID
    assert "at least 2 levels" in err.value.message


def test_vadv_global_variant_requires_scratch(lib):
    t = _native.tune(variant=_native.VADV_GLOBAL)
    with pytest.raises(_native.SbError) as err:
        _run_vadv((8, 4, 3), (1, 1, 0), tune=t)
    assert err.value.code == _native.SB_ERR_INVALID


# ---------------------------------------------------------------------------
# basic stencils beyond the golden cases
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("storage,compute", FORMS)
@pytest.mark.parametrize("along", [(True, True, False), (True, True, True), (False, False, True), (False,) * 3])
def test_laplacian_forms(storage, compute, along, lib):
    domain, halo = (37, 19, 6), (1, 1, 1)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(21, shape, ("inp", "out"), {})
    hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    kernels.laplacian(dev["inp"], dev["out"], along, compute=compute)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = round_to_storage(ora.laplacian(compute_view(hosts["inp"], storage, compute), domain, halo, along), storage)
    _assert_bits(got, want, f"laplacian {along} {storage}/{compute}")


LAP_SHAPES = [
    {"variant": _native.BASIC_POINT},
    {"variant": _native.BASIC_MARCH},
    {"variant": _native.BASIC_MARCH, "tile_y": 4, "block_y": 2},
    {"variant": _native.BASIC_MARCH, "tile_y": 8, "block_y": 8},
    {"variant": _native.BASIC_MARCH, "tile_y": 8, "k_per_cta": 2, "block_y": 1},
]


@pytest.mark.parametrize("storage,compute", FORMS)
@pytest.mark.parametrize("mask", range(1, 8))
@pytest.mark.parametrize("shape", range(len(LAP_SHAPES)))
def test_laplacian_variants(storage, compute, mask, shape, lib):
    """Every Laplacian kernel shape, every axis set, a ragged domain (partial
    warps along i, a partial strip along j, partial k-plane groups): bit-identical
    to the oracle."""
    along = tuple(bool(mask >> a & 1) for a in range(3))
    domain, halo = (37, 19, 7), (1, 1, 1)
    shape_ = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(40 + mask, shape_, ("inp", "out"), {})
    hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    kernels.laplacian(dev["inp"], dev["out"], along, compute=compute, tune=_native.tune(**LAP_SHAPES[shape]))
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    want = round_to_storage(ora.laplacian(compute_view(hosts["inp"], storage, compute), domain, halo, along), storage)
    _assert_bits(got, want, f"laplacian {LAP_SHAPES[shape]} {along} {storage}/{compute}")


@pytest.mark.parametrize("storage", ["float64", "float32"])
@pytest.mark.parametrize("preset", [1, 2, 3, 4])
@pytest.mark.parametrize("special", [False, True])
def test_laplacian_float64_placements(storage, preset, special, lib):
    """float64 Laplacian strips with their subtractions/addition split between
    the fp64 and the integer pipes: the same bits as the oracle, signed zeros
    and cancellations included; with `special`, a sprinkling of subnormal,
    huge, infinite and NaN inputs that the integer path declines (those strips
    are recomputed on the fp64 pipe)."""
    domain, halo = (64, 33, 5), (1, 1, 1)
    shape_ = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(77, shape_, ("inp", "out"), {})
    vals["inp"][::3, ::2, :] = 0.0  # exact cancellations and zero sums
    vals["inp"][1::5, :, ::2] *= -1.0
    if special:
        pick = np.random.Generator(np.random.PCG64(78)).random(size=shape_)
        big = 1e38 if storage == "float32" else 1.5e308
        tiny = 1e-40 if storage == "float32" else 3e-310
        vals["inp"][pick < 0.01] = tiny
        vals["inp"][(pick >= 0.01) & (pick < 0.015)] = -tiny
        vals["inp"][(pick >= 0.015) & (pick < 0.02)] = big
        vals["inp"][(pick >= 0.02) & (pick < 0.022)] = np.inf
        vals["inp"][(pick >= 0.022) & (pick < 0.024)] = np.nan
    hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    t = _native.tune(variant=_native.BASIC_MARCH, flags=preset << 4)
    kernels.laplacian(dev["inp"], dev["out"], (True, True, False), compute="float64", tune=t)
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    with np.errstate(all="ignore"):
        want = round_to_storage(ora.laplacian(compute_view(hosts["inp"], storage, "float64"), domain, halo,
                                              (True, True, False)), storage)
    _assert_bits(got, want, f"laplacian placement {preset} {storage} special={special}")


def test_laplacian_rejects_bad_strip(lib):
    domain, halo = (8, 8, 4), (1, 1, 1)
    shape_ = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(3, shape_, ("inp", "out"), {})
    hosts = {n: host_field(v, "float32", halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float32", halo) for n, h in hosts.items()}
    for bad in ({"tile_y": 5}, {"tile_y": 16}, {"k_per_cta": 4}, {"block_y": 9}, {"flags": 9 << 4}):
        with pytest.raises(_native.SbError) as err:
            kernels.laplacian(dev["inp"], dev["out"], tune=_native.tune(variant=_native.BASIC_MARCH, **bad))
        assert err.value.code == _native.SB_ERR_INVALID


@pytest.mark.parametrize("storage", ["float64", "float32", "bfloat16"])
def test_copy_storage(storage, lib):
    domain, halo = (50, 7, 9), (3, 3, 3)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(22, shape, ("inp", "out"), {})
    hosts = {n: host_field(v, storage, alignment=32, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    kernels.copy(dev["inp"], dev["out"])
    got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
    _assert_bits(got, interior(hosts["inp"], domain, halo), f"copy {storage}")


# ---------------------------------------------------------------------------
# STREAM
# ---------------------------------------------------------------------------


def _fma_exact(b, s, c):
    """Correctly rounded b + s*c for float64 arrays, via exact rationals."""
    from fractions import Fraction

    out = np.empty_like(b)
    for idx in range(b.size):
        exact = Fraction(float(b.flat[idx])) + Fraction(float(s)) * Fraction(float(c.flat[idx]))
        out.flat[idx] = float(exact)
    return out


STREAM_GRIDS = [None, {"variant": _native.STREAM_GRID_STRIDE, "block_x": 512, "unroll": 4},
                {"variant": _native.STREAM_GRID_CHUNK, "block_x": 1024, "unroll": 2},
                {"variant": _native.STREAM_GRID_CHUNK, "block_x": 256, "unroll": 8},
                {"variant": _native.STREAM_GRID_CHUNK, "block_x": 96, "unroll": 1}]


@pytest.mark.parametrize("grid", range(len(STREAM_GRIDS)))
@pytest.mark.parametrize("n,offset", [(1 << 16, 0), ((1 << 16) + 3, 0), (1000, 1), (5, 0)])
def test_stream_ops(n, offset, grid, lib):
    from stencil_benchmarks_gb300.device import DeviceBuffer, copy_to_device, copy_to_host

    rng = np.random.Generator(np.random.PCG64(31))
    bufs = [DeviceBuffer((n + offset) * 8) for _ in range(3)]
    ptrs = [b.ptr + offset * 8 for b in bufs]
    a0, b0, c0 = (rng.random(n) for _ in range(3))

    def put(p, x):
        copy_to_device(p, np.ascontiguousarray(x))

    def get(p):
        x = np.empty(n)
        copy_to_host(x, p)
        return x

    t = _native.tune(**STREAM_GRIDS[grid]) if STREAM_GRIDS[grid] else None
    for p, x in zip(ptrs, (a0, b0, c0)):
        put(p, x)
    kernels.stream_op(_native.STREAM_COPY, "float64", *ptrs, n, tune=t)
    assert np.array_equal(get(ptrs[2]), a0)
    put(ptrs[2], c0)
    kernels.stream_op(_native.STREAM_SCALE, "float64", *ptrs, n, 3.0, tune=t)
    assert bits_equal(get(ptrs[1]), 3.0 * c0)
    put(ptrs[1], b0)
    kernels.stream_op(_native.STREAM_ADD, "float64", *ptrs, n, tune=t)
    assert bits_equal(get(ptrs[2]), a0 + b0)
    put(ptrs[2], c0)
    kernels.stream_op(_native.STREAM_TRIAD, "float64", *ptrs, n, 3.0, tune=t)
    got = get(ptrs[0])
    sample = slice(0, min(n, 2000))
    assert bits_equal(got[sample], _fma_exact(b0[sample], 3.0, c0[sample]))
    assert np.all(np.abs(got - (b0 + 3.0 * c0)) <= np.spacing(b0 + 3.0 * c0))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_stream_reference_sequence(dtype, lib, golden):
    """init + 10 rounds of copy/scale/add/triad give the reference's scalars."""
    from stencil_benchmarks_gb300.device import DeviceBuffer, copy_to_host

    n = (1 << 18) + 5
    item = 8 if dtype == "float64" else 4
    bufs = [DeviceBuffer(n * item) for _ in range(3)]
    a, b, c = (x.ptr for x in bufs)
    kernels.stream_op(_native.STREAM_INIT, dtype, a, b, c, n)
    for _ in range(10):
        for op in (_native.STREAM_COPY, _native.STREAM_SCALE, _native.STREAM_ADD, _native.STREAM_TRIAD):
            kernels.stream_op(op, dtype, a, b, c, n, 3.0)
    want = golden["_stream_scalars"][f"{dtype}_10"]
    # the reference's own criterion (stream/cuda_hip.j2:290-327): average
    # absolute error over the array, relative to the expected value, below
    # 1e-6 (fp32) or 1e-13 (fp64).  fp64 values stay exact integers here.
    eps = 1e-6 if dtype == "float32" else 1e-13
    for ptr, w in zip((a, b, c), want):
        host = np.empty(n, dtype=dtype)
        copy_to_host(host, ptr)
        avg_err = np.mean(np.abs(host.astype(np.float64) - w))
        assert avg_err / abs(w) <= eps
        if dtype == "float64":
            assert np.all(host == w)


# ---------------------------------------------------------------------------
# the full-size workload (512 x 512 x 80, fp64)
# ---------------------------------------------------------------------------


def test_hdiff_full_size_fp64(lib):
    got, want, _ = _run_hdiff((512, 512, 80), (2, 2, 0), seed=101)
    _assert_bits(got, want, "hdiff 512x512x80")


def test_vadv_full_size_fp64_against_c_oracle(lib):
    from oracle import cport

    domain, halo = (512, 512, 80), (1, 1, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(102, shape, VADV_ARGS, VADV_DISTS)
    hosts = {n: host_field(v, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"])
    got = interior(download_like(dev["utensstage"], hosts["utensstage"]), domain, halo)
    cport.vadv(hosts["ustage"], hosts["upos"], hosts["utens"], hosts["utensstage"], hosts["wcon"], domain, halo)
    _assert_bits(got, interior(hosts["utensstage"], domain, halo), "vadv 512x512x80")


@pytest.mark.parametrize("nbytes,offset", [(1 << 20, 0), (12345, 0), (4096 + 7, 3), (16, 0), (1, 0)])
def test_memcpy_sm(nbytes, offset, lib):
    """sb_memcpy_sm between page-locked host and device memory, both ways and
    device to device, with unaligned starts and ragged tails."""
    import ctypes

    from stencil_benchmarks_gb300.device import DeviceBuffer, PinnedBuffer

    rng = np.random.Generator(np.random.PCG64(nbytes))
    src = PinnedBuffer(nbytes + 32)
    src.array(np.uint8, (nbytes + 32,))[...] = rng.integers(0, 256, size=nbytes + 32, dtype=np.uint8)
    dev_a, dev_b = DeviceBuffer(nbytes + 32), DeviceBuffer(nbytes + 32)
    back = PinnedBuffer(nbytes + 32)
    back.array(np.uint8, (nbytes + 32,))[...] = 0
    for dst, s in ((dev_a.ptr + offset, src.ptr + offset), (dev_b.ptr, dev_a.ptr + offset),
                   (back.ptr + offset, dev_b.ptr)):
        _native.call("sb_memcpy_sm", ctypes.c_void_p(dst), ctypes.c_void_p(s), ctypes.c_size_t(nbytes), None)
    _native.synchronize()
    want = src.array(np.uint8, (nbytes + 32,))[offset:offset + nbytes]
    got = back.array(np.uint8, (nbytes + 32,))
    assert np.array_equal(got[offset:offset + nbytes], want)
    assert not got[:offset].any() and not got[offset + nbytes:].any()


def _run_vadv3(domain, halo, storage, compute, tune=None, seed=0, use_scratch=False):
    """sb_vadv3 on u, v, w fields sharing one wcon; returns (got, want) lists."""
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    names = [f"{c}{n}" for c in "uvw" for n in ("stage", "pos", "tens", "tensstage")] + ["wcon"]
    dists = {n: (-1.0, 1.0) for n in names}
    dists["wcon"] = (-0.5, 0.5)
    vals = rng_fields(seed, shape, names, dists)
    hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    scratch = {}
    if use_scratch:
        for n in ("ccol", "dcol"):
            hosts[n] = host_field(np.zeros(shape), "float64" if compute == "float64" else storage, halo=halo)
            scratch[n] = to_device(hosts[n], "float64" if compute == "float64" else storage, halo)
    comps = [tuple(dev[f"{c}{n}"] for n in ("stage", "pos", "tens", "tensstage")) for c in "uvw"]
    outs = []
    for c in "uvw":
        hosts[f"{c}out"] = host_field(np.zeros(shape), storage, halo=halo)
        dev[f"{c}out"] = to_device(hosts[f"{c}out"], storage, halo)
        outs.append(dev[f"{c}out"])
    kernels.vadv3(comps, dev["wcon"], outs=outs, compute=compute, tune=tune, **scratch)
    _native.synchronize()
    got, want = [], []
    oracle = "float64" if compute == "float32x2" else compute  # float pairs against the float64 oracle
    for c, shift in zip("uvw", ((1, 0), (0, 1), (0, 0))):
        got.append(interior(download_like(dev[f"{c}out"], hosts[f"{c}out"]), domain, halo))
        f = {n: compute_view(hosts[f"{c}{n}"], storage, oracle) for n in ("stage", "pos", "tens", "tensstage")}
        with np.errstate(all="ignore"):
            comp = ora._vadv_component(f["stage"], f["pos"], f["tens"], f["tensstage"],
                                       compute_view(hosts["wcon"], storage, oracle), domain, halo, *shift)
        want.append(round_to_storage(comp, storage))
    # the in-place inputs are untouched when outputs go elsewhere
    return got, want


@pytest.mark.parametrize("storage,compute,tune,domain", [
    ("float32", "float32", {"variant": _native.VADV_TMEM}, (70, 33, 17)),    # fused, explicit, ragged
    ("bfloat16", "float32", {"variant": _native.VADV_TMEM}, (64, 20, 9)),    # fused, 2-byte storage
    ("float32", "float32", None, (128, 512, 12)),                            # fused under AUTO (2048 groups)
    ("float32", "float32", None, (40, 30, 11)),                               # AUTO, small: three launches
    ("float64", "float64", None, (45, 20, 13)),                               # three launches, exact fp64
    ("float64", "float32x2", None, (33, 17, 7)),                              # three launches, float pair
])
def test_vadv3_all_components(storage, compute, tune, domain, lib):
    """sb_vadv3 (u, v, w on one wcon; fused into one launch where the
    tensor-memory form applies): every component bit-identical to the oracle,
    or within the float-pair tolerance."""
    t = _native.tune(**tune) if tune else None
    got, want = _run_vadv3(domain, (1, 1, 1), storage, compute, tune=t, seed=sum(domain),
                           use_scratch=compute == "float32x2")
    for c, g, w in zip("uvw", got, want):
        if compute == "float32x2":
            scale = np.max(np.abs(w))
            assert np.max(np.abs(g - w)) <= 1e-9 * scale, f"vadv3 {c} {storage}/{compute}"
        else:
            _assert_bits(g, w, f"vadv3 {c} {storage}/{compute} {tune}")


def test_stream_rejects_bad_grid(lib):
    from stencil_benchmarks_gb300.device import DeviceBuffer

    bufs = [DeviceBuffer(64 * 8) for _ in range(3)]
    for bad in ({"variant": 3}, {"variant": _native.STREAM_GRID_STRIDE, "block_x": 1024},
                {"variant": _native.STREAM_GRID_CHUNK, "block_x": 2048},
                {"variant": _native.STREAM_GRID_CHUNK, "unroll": 3}):
        with pytest.raises(_native.SbError) as err:
            kernels.stream_op(_native.STREAM_COPY, "float64", *(b.ptr for b in bufs), 64, tune=_native.tune(**bad))
        assert err.value.code == _native.SB_ERR_INVALID
