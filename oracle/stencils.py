"""Numpy restatement of the reference's stencil verification arithmetic.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the product package never
imports this module.

Every function takes the full halo'd arrays exactly as the reference allocates
them (shape ``domain + 2*halo``, any strides) and returns the expected values
of the output field on the interior (shape ``domain``).  The operation order
and the dtype of every intermediate follow the reference so that results are
bit-identical to what ``verify_stencil`` compares against:

* numpy 2 treats Python scalars as "weak", so ``4 * inp`` or ``3 / 20 * x``
  stays in the array's dtype -- a float32 oracle computes in float32;
* no operation is fused (numpy rounds after every ``+ - * /``).

Sources (paths inside the reference project):
  copy        stencil_benchmarks/benchmarks_collection/stencils/base.py:180-188
  averages    .../stencils/base.py:191-222
  Laplacian   .../stencils/base.py:225-254
  hdiff       .../stencils/base.py:276-311  (same order as numpy/horizontal_diffusion.py:42-56)
  vadv        .../stencils/base.py:349-501
  STREAM      stencil_benchmarks/benchmarks_collection/stream/cuda_hip.j2:132-173, 329-345
"""

from __future__ import annotations

import numpy as np


def inner_slice(domain, halo, shift=None):
    """Index of the interior, optionally shifted (base.py:127-137)."""
    shift = (0, 0, 0) if shift is None else shift
    return tuple(slice(h + s, h + d + s) for d, h, s in zip(domain, halo, shift))


# ----------------------------------------------------------------------------
# basic stencils
# ----------------------------------------------------------------------------


def copy(inp, domain, halo):
    """out = inp on the interior (base.py:180-188)."""
    return inp[inner_slice(domain, halo)].copy()


def onesided_average(inp, domain, halo, axis):
    """out = (inp[+1] + inp) / 2 along ``axis`` (base.py:191-205)."""
    shift = [0, 0, 0]
    shift[axis] = 1
    return (inp[inner_slice(domain, halo, shift)] + inp[inner_slice(domain, halo)]) / 2


def symmetric_average(inp, domain, halo, axis):
    """out = (inp[+1] + inp[-1]) / 2 along ``axis`` (base.py:208-222)."""
    shift = [0, 0, 0]
    shift[axis] = 1
    neg = [-s for s in shift]
    return (inp[inner_slice(domain, halo, shift)] + inp[inner_slice(domain, halo, neg)]) / 2


def laplacian(inp, domain, halo, along=(True, True, False)):
    """Sum over the chosen axes of 2*inp - inp[+1] - inp[-1] (base.py:238-254).

    The accumulator starts at zero and the axis terms are added in x, y, z
    order, exactly as the reference does.
    """
    result = np.zeros(tuple(domain), dtype=inp.dtype)
    center = inp[inner_slice(domain, halo)]
    for axis, use in enumerate(along):
        if use:
            shift = [0, 0, 0]
            shift[axis] = 1
            neg = [-s for s in shift]
            result += (
                2 * center
                - inp[inner_slice(domain, halo, shift)]
                - inp[inner_slice(domain, halo, neg)]
            )
    return result


# ----------------------------------------------------------------------------
# horizontal diffusion
# ----------------------------------------------------------------------------


def hdiff(inp, coeff, domain, halo):
    """Horizontal diffusion with flux limiter (base.py:276-311).

    lap = 4*inp - (((inp[i+1] + inp[i-1]) + inp[j+1]) + inp[j-1])
    flx = lap[i+1] - lap[i], set to 0 where flx * (inp[i+1] - inp[i]) > 0
    fly = lap[j+1] - lap[j], set to 0 where fly * (inp[j+1] - inp[j]) > 0
    out = inp - coeff * (((flx[i] - flx[i-1]) + fly[j]) - fly[j-1])
    """
    lap = np.zeros_like(inp)
    lap[1:-1, 1:-1, :] = 4 * inp[1:-1, 1:-1, :] - (
        inp[2:, 1:-1, :] + inp[:-2, 1:-1, :] + inp[1:-1, 2:, :] + inp[1:-1, :-2, :]
    )

    flx = np.zeros_like(inp)
    flx[:-1, :, :] = lap[1:, :, :] - lap[:-1, :, :]
    flx[:-1, :, :] = np.where(
        flx[:-1, :, :] * (inp[1:, :, :] - inp[:-1, :, :]) > 0, 0, flx[:-1, :, :]
    )

    fly = np.zeros_like(inp)
    fly[:, :-1, :] = lap[:, 1:, :] - lap[:, :-1, :]
    fly[:, :-1, :] = np.where(
        fly[:, :-1, :] * (inp[:, 1:, :] - inp[:, :-1, :]) > 0, 0, fly[:, :-1, :]
    )

    result = np.zeros_like(inp)
    result[1:-1, 1:-1, :] = inp[1:-1, 1:-1, :] - coeff[1:-1, 1:-1, :] * (
        flx[1:-1, 1:-1, :] - flx[:-2, 1:-1, :] + fly[1:-1, 1:-1, :] - fly[1:-1, :-2, :]
    )
    return result[inner_slice(domain, halo)]


def hdiff_limiter_stats(inp, coeff, domain, halo):
    """Count limiter decisions that sit exactly on the ``> 0`` boundary.

    Returns ``(exact_zero_products, total_fluxes)`` over the fluxes that feed
    interior outputs: a product of exactly 0 is where a reduced-precision input
    can flip the branch.
    """
    hi, hj, _ = halo
    ni, nj, _ = domain
    sl = inner_slice(domain, halo)
    lap = np.zeros_like(inp)
    lap[1:-1, 1:-1, :] = 4 * inp[1:-1, 1:-1, :] - (
        inp[2:, 1:-1, :] + inp[:-2, 1:-1, :] + inp[1:-1, 2:, :] + inp[1:-1, :-2, :]
    )
    zeros = 0
    total = 0
    # fluxes used by the interior: flx at i-1..ni-1, fly at j-1..nj-1
    fx = (slice(hi - 1, hi + ni), sl[1], sl[2])
    fxp = (slice(hi, hi + ni + 1), sl[1], sl[2])
    flx = lap[fxp] - lap[fx]
    prod = flx * (inp[fxp] - inp[fx])
    zeros += int(np.count_nonzero(prod == 0))
    total += prod.size
    fy = (sl[0], slice(hj - 1, hj + nj), sl[2])
    fyp = (sl[0], slice(hj, hj + nj + 1), sl[2])
    fly = lap[fyp] - lap[fy]
    prod = fly * (inp[fyp] - inp[fy])
    zeros += int(np.count_nonzero(prod == 0))
    total += prod.size
    return zeros, total


# ----------------------------------------------------------------------------
# vertical advection
# ----------------------------------------------------------------------------

DTR_STAGE = 3 / 20
BETA_V = 0
BET_M = 0.5 * (1 - BETA_V)
BET_P = 0.5 * (1 + BETA_V)


def _vadv_component(stage, pos, tens, tensstage, wcon, domain, halo, ishift, jshift):
    """Thomas solve of one velocity component (base.py:415-473).

    Works on (ni, nj) planes with a Python loop over k, in the dtype of the
    input arrays.  Returns the new ``tensstage`` interior.
    """
    hi, hj, hk = halo
    ni, nj, nk = domain
    if nk < 2:
        raise ValueError("vertical advection needs at least 2 levels")

    def plane(a, k, di=0, dj=0):
        return a[hi + di : hi + di + ni, hj + dj : hj + dj + nj, hk + k]

    dtype = stage.dtype
    ccol = np.empty((ni, nj, nk), dtype=dtype)
    dcol = np.empty((ni, nj, nk), dtype=dtype)
    dtr_stage = DTR_STAGE

    # forward sweep, k = 0
    k = 0
    gcv = 0.25 * (plane(wcon, k + 1, ishift, jshift) + plane(wcon, k + 1))
    cs = gcv * BET_M
    ccol[:, :, k] = gcv * BET_P
    bcol = dtr_stage - ccol[:, :, k]
    correction_term = -cs * (plane(stage, k + 1) - plane(stage, k))
    dcol[:, :, k] = (
        dtr_stage * plane(pos, k) + plane(tens, k) + plane(tensstage, k) + correction_term
    )
    ccol[:, :, k] /= bcol
    dcol[:, :, k] /= bcol

    for k in range(1, nk - 1):
        gav = -0.25 * (plane(wcon, k, ishift, jshift) + plane(wcon, k))
        gcv = 0.25 * (plane(wcon, k + 1, ishift, jshift) + plane(wcon, k + 1))
        as_ = gav * BET_M
        cs = gcv * BET_M
        acol = gav * BET_P
        ccol[:, :, k] = gcv * BET_P
        bcol = dtr_stage - acol - ccol[:, :, k]
        correction_term = -as_ * (plane(stage, k - 1) - plane(stage, k)) - cs * (
            plane(stage, k + 1) - plane(stage, k)
        )
        dcol[:, :, k] = (
            dtr_stage * plane(pos, k) + plane(tens, k) + plane(tensstage, k) + correction_term
        )
        divided = 1.0 / (bcol - ccol[:, :, k - 1] * acol)
        ccol[:, :, k] *= divided
        dcol[:, :, k] = (dcol[:, :, k] - dcol[:, :, k - 1] * acol) * divided

    k = nk - 1
    gav = -0.25 * (plane(wcon, k, ishift, jshift) + plane(wcon, k))
    as_ = gav * BET_M
    acol = gav * BET_P
    bcol = dtr_stage - acol
    correction_term = -as_ * (plane(stage, k - 1) - plane(stage, k))
    dcol[:, :, k] = (
        dtr_stage * plane(pos, k) + plane(tens, k) + plane(tensstage, k) + correction_term
    )
    dcol[:, :, k] = (dcol[:, :, k] - dcol[:, :, k - 1] * acol) / (
        bcol - ccol[:, :, k - 1] * acol
    )

    # backward sweep
    out = np.empty((ni, nj, nk), dtype=dtype)
    k = nk - 1
    datacol = dcol[:, :, k]
    out[:, :, k] = dtr_stage * (datacol - plane(pos, k))
    for k in range(nk - 2, -1, -1):
        datacol = dcol[:, :, k] - ccol[:, :, k] * datacol
        out[:, :, k] = dtr_stage * (datacol - plane(pos, k))
    return out


def vadv(fields, domain, halo, all_components=False):
    """Vertical advection oracle (base.py:349-501).

    ``fields`` maps the reference's argument names (``ustage``, ``upos``,
    ``utens``, ``utensstage``, ``wcon`` and, with ``all_components``, the v and
    w fields) to halo'd arrays.  Returns a dict ``{"utensstage": ...}`` (plus
    ``vtensstage`` / ``wtensstage``) of expected interiors.  The u component
    reads wcon at i+1, v at j+1, w at the same column (base.py:475-483).
    """
    out = {
        "utensstage": _vadv_component(
            fields["ustage"], fields["upos"], fields["utens"], fields["utensstage"],
            fields["wcon"], domain, halo, 1, 0,
        )
    }
    if all_components:
        out["vtensstage"] = _vadv_component(
            fields["vstage"], fields["vpos"], fields["vtens"], fields["vtensstage"],
            fields["wcon"], domain, halo, 0, 1,
        )
        out["wtensstage"] = _vadv_component(
            fields["wstage"], fields["wpos"], fields["wtens"], fields["wtensstage"],
            fields["wcon"], domain, halo, 0, 0,
        )
    return out


# ----------------------------------------------------------------------------
# STREAM
# ----------------------------------------------------------------------------


def stream_copy(a):
    """c = a (cuda_hip.j2:141-144)."""
    return a.copy()


def stream_scale(c, scalar):
    """b = scalar * c (cuda_hip.j2:146-150)."""
    return (c.dtype.type(scalar) * c).astype(c.dtype)


def stream_add(a, b):
    """c = a + b (cuda_hip.j2:152-156)."""
    return a + b


def stream_triad(b, c, scalar):
    """a = b + scalar * c with two roundings (numpy); cuda_hip.j2:158-163.

    The GPU kernels (the reference's and ours) evaluate this with one fused
    multiply-add, which differs from this value by at most one ulp.
    """
    return b + c.dtype.type(scalar) * c


def stream_expected_scalars(ntimes, dtype="float64", scalar=3):
    """Values a, b, c hold after ``ntimes`` rounds of copy/scale/add/triad
    starting from a=1, b=2, c=0 (cuda_hip.j2:329-345)."""
    t = np.dtype(dtype).type
    aj, bj, cj, s = t(1), t(2), t(0), t(scalar)
    for _ in range(ntimes):
        cj = aj
        bj = s * cj
        cj = aj + bj
        aj = bj + s * cj
    return aj, bj, cj


# ----------------------------------------------------------------------------
# reduced-precision storage helpers
# ----------------------------------------------------------------------------


def f32_to_bf16_bits(x):
    """Round float32 values to bfloat16 (round to nearest, ties to even).

    Returns the 16-bit patterns as uint16.  NaNs stay NaN (quiet bit set).
    """
    x = np.ascontiguousarray(x, dtype=np.float32)
    bits = x.view(np.uint32).astype(np.uint64)
    lsb = (bits >> 16) & 1
    rounded = ((bits + 0x7FFF + lsb) >> 16).astype(np.uint16)
    nan = np.isnan(x)
    if np.any(nan):
        rounded = np.where(nan, ((bits >> 16) | 0x40).astype(np.uint16), rounded)
    return rounded


def bf16_bits_to_f32(b):
    """Widen bfloat16 bit patterns (uint16) to float32 exactly."""
    b = np.ascontiguousarray(b, dtype=np.uint16)
    return (b.astype(np.uint32) << 16).view(np.float32)


def quantize(x, storage):
    """Return ``x`` as it reads back after a round trip through ``storage``.

    storage is "float64", "float32" or "bfloat16"; the result is float64 for
    float64 storage and float32 otherwise (the compute type of that form).
    """
    if storage == "float64":
        return np.asarray(x, dtype=np.float64)
    if storage == "float32":
        return np.asarray(x, dtype=np.float32)
    if storage == "bfloat16":
        return bf16_bits_to_f32(f32_to_bf16_bits(np.asarray(x, dtype=np.float32))).reshape(
            np.shape(x)
        )
    raise ValueError(f"unknown storage type {storage!r}")
