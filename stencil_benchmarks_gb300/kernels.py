"""Python wrappers of the stencil entry points, taking ``device.Field`` objects.

Each function launches one kernel on ``stream`` (default stream if None).
With ``timed=True`` the call waits for the kernel and returns its duration in
seconds measured with CUDA events (the reference's "gpu" timers); otherwise
it returns None immediately after the asynchronous launch.
"""

from __future__ import annotations

import ctypes

from . import _native
from .device import Field, _stream_arg


def _check_same_layout(*fields: Field):
    first = fields[0]
    for f in fields[1:]:
        if f.strides != first.strides or f.storage != first.storage:
            raise ValueError("all fields of a stencil must share strides and storage type")
        if f.halo != first.halo or f.shape != first.shape:
            raise ValueError("all fields of a stencil must share shape and halo")


def _compute_code(storage: str, compute: str | None) -> int:
    if compute is None or compute == "auto":
        return _native.SB_F64 if storage == "float64" else _native.SB_F32
    return _native.storage_code(compute)


def _domain(field: Field):
    return tuple(n - 2 * h for n, h in zip(field.shape, field.halo))


def _tune_arg(tune):
    if tune is None:
        return None
    if isinstance(tune, dict):
        tune = _native.tune(**tune)
    return ctypes.byref(tune)


def _launch(name, args, timed):
    t = _native.timed_out() if timed else None
    _native.call(name, *args, ctypes.byref(t) if timed else None)
    return t.value if timed else None


def hdiff(inp: Field, coeff: Field, out: Field, compute=None, tune=None, stream=None, timed=False):
    """out = horizontal_diffusion(inp, coeff) on the interior; halo >= 2 in i, j."""
    _check_same_layout(inp, coeff, out)
    if min(inp.halo[:2]) < 2:
        raise ValueError(f"horizontal diffusion needs a halo of at least 2 in i and j (got {inp.halo})")
    ni, nj, nk = _domain(inp)
    args = [
        _native.storage_code(inp.storage), _compute_code(inp.storage, compute),
        ctypes.c_void_p(inp.interior_ptr), ctypes.c_void_p(coeff.interior_ptr), ctypes.c_void_p(out.interior_ptr),
        ni, nj, nk, *inp.strides, _tune_arg(tune), _stream_arg(stream),
    ]
    return _launch("sb_hdiff", args, timed)


def vadv(stage: Field, pos: Field, tens: Field, tensstage: Field, wcon: Field, shift=(1, 0),
         ccol: Field | None = None, dcol: Field | None = None, out: Field | None = None, compute=None,
         tune=None, stream=None, timed=False):
    """Thomas solve of one component; wcon is read at ``shift``.

    The new tensstage goes to ``out`` (default: ``tensstage`` itself, the
    reference's in-place update)."""
    out = tensstage if out is None else out
    _check_same_layout(stage, pos, tens, tensstage, wcon, out)
    need = [h >= s for h, s in zip(stage.halo[:2], shift)]
    if not all(need):
        raise ValueError(f"vertical advection needs a halo >= 1 along the wcon shift {shift} (got {stage.halo})")
    for scratch in (ccol, dcol):
        if scratch is not None and scratch.strides != stage.strides:
            raise ValueError("ccol/dcol scratch fields must have the same strides as the other fields")
    ni, nj, nk = _domain(stage)
    args = [
        _native.storage_code(stage.storage), _compute_code(stage.storage, compute),
        *(ctypes.c_void_p(f.interior_ptr) for f in (stage, pos, tens, tensstage, wcon, out)),
        ctypes.c_void_p(ccol.interior_ptr) if ccol is not None else None,
        ctypes.c_void_p(dcol.interior_ptr) if dcol is not None else None,
        ni, nj, nk, *stage.strides, int(shift[0]), int(shift[1]), _tune_arg(tune), _stream_arg(stream),
    ]
    return _launch("sb_vadv", args, timed)


def vadv3(components, wcon: Field, ccol: Field | None = None, dcol: Field | None = None, outs=None, compute=None,
          tune=None, stream=None, timed=False):
    """All three components, u, v, w, on one wcon (wcon read at (1, 0), (0, 1)
    and (0, 0)): ``components`` = three (stage, pos, tens, tensstage) tuples;
    the new tensstages go to ``outs`` (default: the tensstages in place).  One
    fused launch where the tensor-memory form applies (float32 compute), else
    one launch per component."""
    comps = [tuple(c) for c in components]
    if len(comps) != 3 or any(len(c) != 4 for c in comps):
        raise ValueError("vadv3 takes three (stage, pos, tens, tensstage) tuples")
    outs = [c[3] for c in comps] if outs is None else list(outs)
    fields = [f for c in comps for f in c] + [wcon] + outs
    _check_same_layout(*fields)
    if any(h < 1 for h in wcon.halo[:2]):
        raise ValueError(f"vertical advection of u and v needs a halo >= 1 along i and j (got {wcon.halo})")
    for scratch in (ccol, dcol):
        if scratch is not None and scratch.strides != wcon.strides:
            raise ValueError("ccol/dcol scratch fields must have the same strides as the other fields")
    ni, nj, nk = _domain(wcon)
    arr = ctypes.c_void_p * 3

    def ptrs(k):
        return arr(*(c[k].interior_ptr for c in comps))

    args = [
        _native.storage_code(wcon.storage), _compute_code(wcon.storage, compute),
        ptrs(0), ptrs(1), ptrs(2), ptrs(3), ctypes.c_void_p(wcon.interior_ptr), arr(*(o.interior_ptr for o in outs)),
        ctypes.c_void_p(ccol.interior_ptr) if ccol is not None else None,
        ctypes.c_void_p(dcol.interior_ptr) if dcol is not None else None,
        ni, nj, nk, *wcon.strides, _tune_arg(tune), _stream_arg(stream),
    ]
    return _launch("sb_vadv3", args, timed)


def copy(inp: Field, out: Field, tune=None, stream=None, timed=False):
    _check_same_layout(inp, out)
    ni, nj, nk = _domain(inp)
    args = [_native.storage_code(inp.storage), ctypes.c_void_p(inp.interior_ptr), ctypes.c_void_p(out.interior_ptr),
            ni, nj, nk, *inp.strides, _tune_arg(tune), _stream_arg(stream)]
    return _launch("sb_copy", args, timed)


def empty(field: Field, tune=None, stream=None, timed=False):
    """The empty kernel over ``field``'s interior grid (launch overhead)."""
    ni, nj, nk = _domain(field)
    return _launch("sb_empty", [ni, nj, nk, _tune_arg(tune), _stream_arg(stream)], timed)


def laplacian(inp: Field, out: Field, along=(True, True, False), compute=None, tune=None, stream=None,
              timed=False):
    _check_same_layout(inp, out)
    ni, nj, nk = _domain(inp)
    mask = sum(1 << a for a, use in enumerate(along) if use)
    args = [_native.storage_code(inp.storage), _compute_code(inp.storage, compute),
            ctypes.c_void_p(inp.interior_ptr), ctypes.c_void_p(out.interior_ptr),
            ni, nj, nk, *inp.strides, mask, _tune_arg(tune), _stream_arg(stream)]
    return _launch("sb_laplacian", args, timed)


def average(inp: Field, out: Field, axis: int, symmetric: bool, compute=None, tune=None, stream=None,
            timed=False):
    _check_same_layout(inp, out)
    ni, nj, nk = _domain(inp)
    args = [_native.storage_code(inp.storage), _compute_code(inp.storage, compute),
            ctypes.c_void_p(inp.interior_ptr), ctypes.c_void_p(out.interior_ptr),
            ni, nj, nk, *inp.strides, int(axis), int(bool(symmetric)), _tune_arg(tune), _stream_arg(stream)]
    return _launch("sb_average", args, timed)


def stream_op(op: int, dtype: str, a: int, b: int, c: int, n: int, scalar: float = 3.0, tune=None,
              stream=None, timed=False):
    """STREAM op on raw device pointers a, b, c of n elements each."""
    args = [int(op), _native.storage_code(dtype), ctypes.c_void_p(a), ctypes.c_void_p(b), ctypes.c_void_p(c),
            float(scalar), int(n), _tune_arg(tune), _stream_arg(stream)]
    return _launch("sb_stream_op", args, timed)


def arith_rate(kind: int) -> float:
    """Measured operations per second: 0 fp64 add, 1 fp64 fma, 2 fp32 fma, 3 f64->f32
    conversion, 4 f32->f64 conversion, 5 32-bit integer shift/xor/multiply, 6 u32->f32
    conversion, 7 s32->f32 conversion, 8 / 9 fp64 add / multiply in integer arithmetic,
    10 fp64 adds beside independent integer work, 11 that integer work alone, 12 / 13 the
    fp64 reciprocal in integer arithmetic / as the fp64 sequence, 14 / 15 the 64-bit
    leading-zero count as the instruction / from a conversion, 16 / 17 those beside one
    fp64 add each, 18 / 19 / 20 fp64 adds beside an integer binary64 add / a 64-bit variable
    shift / a 64-bit add and compare (see sb_probe_arith_rate)."""
    out = ctypes.c_double()
    _native.call("sb_probe_arith_rate", int(kind), ctypes.byref(out))
    return out.value
