"""ctypes binding of ``libsbgb300.so`` (declared in ``include/sbgb300.h``).

The library is built in-tree (``python -m stencil_benchmarks_gb300.build``).
There is no fallback: if the library is missing or fails to load, every
entry point raises ``NativeLibraryError``.  A failing call raises
``SbError`` carrying the library's own message (``sb_last_error``), the
counterpart of the reference's ``ExecutionError`` built from the generated
launcher's stderr (stencil_benchmarks/tools/compilation.py:176-193).
"""

from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

import numpy as np

LIBRARY = Path(__file__).resolve().parent / "libsbgb300.so"

SB_OK = 0
SB_ERR_INVALID = 1
SB_ERR_CUDA = 2
SB_ERR_UNSUPPORTED = 3
SB_ERR_NOMEM = 4
SB_ERR_TIMEOUT = 5
SB_ERR_BUDGET = 6
SB_NOT_READY = 7

SB_F64, SB_F32, SB_BF16 = 0, 1, 2
SB_F32X2 = 3  # compute only: float pair ("double-float") with float64 storage
SB_FIX64 = 4  # compute only (hdiff): 64-bit fixed-point sums with float64 storage
H2H, H2D, D2H, D2D = 0, 1, 2, 3

STREAM_INIT, STREAM_COPY, STREAM_SCALE, STREAM_ADD, STREAM_TRIAD = range(5)
STREAM_GRID_STRIDE, STREAM_GRID_CHUNK = 1, 2
BASIC_POINT, BASIC_MARCH = 1, 2

VARIANT_AUTO = 0
HDIFF_TILE, HDIFF_JSCAN, HDIFF_TMA, HDIFF_VSCAN = 1, 2, 3, 4
VADV_SMEM, VADV_GLOBAL, VADV_SLAB, VADV_WSLAB, VADV_TMEM = 1, 2, 3, 4, 5

DTYPE_CODES = {"float64": SB_F64, "float32": SB_F32, "bfloat16": SB_BF16, "float32x2": SB_F32X2,
               "fixed64": SB_FIX64}


class NativeLibraryError(RuntimeError):
    """libsbgb300.so is missing or could not be loaded (no CPU fallback exists)."""


class SbError(RuntimeError):
    """A library call returned a non-zero status."""

    def __init__(self, func, code, message):
        self.func = func
        self.code = code
        self.message = message
        super().__init__(f"{func} failed (status {code}): {message}")


class SbTune(ctypes.Structure):
    _fields_ = [
        ("variant", ctypes.c_int32),
        ("block_x", ctypes.c_int32),
        ("block_y", ctypes.c_int32),
        ("tile_y", ctypes.c_int32),
        ("k_per_cta", ctypes.c_int32),
        ("unroll", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


def tune(**kw) -> SbTune:
    t = SbTune()
    for k, v in kw.items():
        setattr(t, k, int(v))
    return t


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double
_size = ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_tp = ctypes.POINTER(SbTune)

# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "sb_last_error": [],
    "sb_version": [],
    "sb_device_count": [ctypes.POINTER(_int)],
    "sb_set_device": [_int],
    "sb_get_device": [ctypes.POINTER(_int)],
    "sb_device_info": [_int, ctypes.c_char_p, _int, ctypes.POINTER(_int), ctypes.POINTER(_int),
                       ctypes.POINTER(_int), ctypes.POINTER(_size), ctypes.POINTER(_int),
                       ctypes.POINTER(_int)],
    "sb_synchronize": [],
    "sb_kernel_status": [],
    "sb_debug_wait_limit": [_int],
    "sb_malloc": [ctypes.POINTER(_vp), _size],
    "sb_free": [_vp],
    "sb_malloc_host": [ctypes.POINTER(_vp), _size],
    "sb_free_host": [_vp],
    "sb_memcpy": [_vp, _vp, _size, _int],
    "sb_memcpy_async": [_vp, _vp, _size, _int, _vp],
    "sb_memcpy_sm": [_vp, _vp, _size, _vp],
    "sb_memset": [_vp, _int, _size],
    "sb_mem_info": [ctypes.POINTER(_size), ctypes.POINTER(_size)],
    "sb_stream_create": [ctypes.POINTER(_vp)],
    "sb_stream_destroy": [_vp],
    "sb_stream_synchronize": [_vp],
    "sb_event_create": [ctypes.POINTER(_vp)],
    "sb_event_destroy": [_vp],
    "sb_event_record": [_vp, _vp],
    "sb_event_elapsed": [_vp, _vp, _dp],
    "sb_event_synchronize": [_vp],
    "sb_l2_flush": [_vp],
    "sb_stream_op": [_int, _int, _vp, _vp, _vp, _dbl, _i64, _tp, _vp, _dp],
    "sb_copy": [_int, _vp, _vp] + [_i64] * 6 + [_tp, _vp, _dp],
    "sb_empty": [_i64] * 3 + [_tp, _vp, _dp],
    "sb_laplacian": [_int, _int, _vp, _vp] + [_i64] * 6 + [_int, _tp, _vp, _dp],
    "sb_average": [_int, _int, _vp, _vp] + [_i64] * 6 + [_int, _int, _tp, _vp, _dp],
    "sb_hdiff": [_int, _int, _vp, _vp, _vp] + [_i64] * 6 + [_tp, _vp, _dp],
    "sb_vadv": [_int, _int] + [_vp] * 8 + [_i64] * 6 + [_int, _int, _tp, _vp, _dp],
    # stage, pos, tens, tensstage: arrays of three pointers; wcon; out: three pointers; ccol, dcol
    "sb_vadv3": [_int, _int] + [ctypes.POINTER(_vp)] * 4 + [_vp, ctypes.POINTER(_vp), _vp, _vp] + [_i64] * 6
                + [_tp, _vp, _dp],
    "sb_vadv_noalloc": [_int, _int] + [_vp] * 6 + [_i64] * 6 + [_int, _int, _vp, _dp],
    # batch entry points take struct pointers; batching.py narrows these types
    "sb_batch_create": [ctypes.POINTER(_vp), _int, _int, _int, _i64, _vp],
    "sb_batch_set": [_vp, _vp, _int],
    "sb_batch_launch": [_vp, _vp, _dp],
    "sb_batch_info": [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_size), ctypes.POINTER(_int),
                      ctypes.POINTER(_int)],
    "sb_batch_destroy": [_vp],
    "sb_fill_batch": [_vp, _int, _vp, _vp],
    "sb_event_query": [_vp],
    "sb_stream_wait_event": [_vp, _vp],
    "sb_arena_create": [ctypes.POINTER(_vp), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64],
    "sb_arena_alloc": [_vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "sb_arena_free": [_vp, ctypes.c_uint64],
    "sb_arena_stats": [_vp] + [ctypes.POINTER(ctypes.c_uint64)] * 4,
    "sb_arena_destroy": [_vp],
    # server entry points take struct pointers (serving.py passes ctypes structures)
    "sb_server_create": [ctypes.POINTER(_vp), _vp],
    "sb_server_destroy": [_vp],
    "sb_server_submit": [_vp, _vp],
    "sb_server_step": [_vp, _dbl, ctypes.POINTER(_int)],
    "sb_server_take_completed": [_vp, _vp, _int, ctypes.POINTER(_int)],
    "sb_server_field": [_vp, _i64, _int, ctypes.POINTER(_vp)],
    "sb_server_query": [_vp, _i64, _vp],
    "sb_server_release": [_vp, _i64],
    "sb_server_stats": [_vp, _vp],
    "sb_server_debug_complete": [_vp],
    "sb_server_debug_launches": [_vp, _vp, _int, ctypes.POINTER(_int)],
    "sb_probe_arith_rate": [_int, _dp],
    "sb_debug_soft_f64": [_int, _vp, _vp, _vp, _i64, _vp],
}
_RESTYPES = {"sb_last_error": ctypes.c_char_p}

_lock = threading.Lock()
_lib = None


def lib():
    """Load the library once; raise NativeLibraryError if it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = Path(os.environ.get("SBGB300_LIBRARY", LIBRARY))
        if not path.exists():
            raise NativeLibraryError(
                f"{path} not found: build it with `python -m stencil_benchmarks_gb300.build` "
                "(there is no CPU fallback)"
            )
        try:
            handle = ctypes.CDLL(str(path))
        except OSError as err:
            raise NativeLibraryError(f"cannot load {path}: {err}") from err
        for name, argtypes in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = handle
        return _lib


def last_error() -> str:
    msg = lib().sb_last_error()
    return msg.decode() if msg else ""


def call(name, *args):
    """Call ``name`` and raise SbError on a non-zero status."""
    rc = getattr(lib(), name)(*args)
    if rc != SB_OK:
        raise SbError(name, rc, last_error())
    return rc


def device_count() -> int:
    n = ctypes.c_int(0)
    call("sb_device_count", ctypes.byref(n))
    return n.value


def current_device() -> int:
    n = ctypes.c_int(0)
    call("sb_get_device", ctypes.byref(n))
    return n.value


def device_info(device: int = 0) -> dict:
    name = ctypes.create_string_buffer(256)
    sm, major, minor, l2, smem = (ctypes.c_int() for _ in range(5))
    total = ctypes.c_size_t()
    call("sb_device_info", device, name, 256, ctypes.byref(sm), ctypes.byref(major),
         ctypes.byref(minor), ctypes.byref(total), ctypes.byref(l2), ctypes.byref(smem))
    return {
        "name": name.value.decode(),
        "sm_count": sm.value,
        "compute_capability": (major.value, minor.value),
        "total_mem": total.value,
        "l2_bytes": l2.value,
        "smem_optin": smem.value,
    }


def synchronize():
    call("sb_synchronize")


def timed_out():
    """A fresh ctypes double for the `time_s` out-parameter."""
    return ctypes.c_double(0.0)


def storage_code(dtype) -> int:
    name = dtype if isinstance(dtype, str) else np.dtype(dtype).name
    try:
        return DTYPE_CODES[name]
    except KeyError:
        raise ValueError(f"unsupported element type {name!r}") from None
