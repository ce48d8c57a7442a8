"""ctypes binding of ``oracle/csrc/oracle.c`` (the C restatement).

TEST INFRASTRUCTURE ONLY: imported by tests/ (second oracle) and by bench.py
(timed CPU baseline, ``cpu_baseline.kind == "port"``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "csrc" / "oracle.c"
LIBRARY = HERE / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the C oracle with gcc (OpenMP, strict IEEE: no contraction)."""
    if LIBRARY.exists() and not force and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIBRARY
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        os.environ.get("CC", "gcc"), "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
        "-std=c11", "-fPIC", "-shared", str(SOURCE), "-o", str(tmp),
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIBRARY)
    return LIBRARY


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIBRARY))
        i64 = ctypes.c_int64
        vp = ctypes.c_void_p
        for sfx in ("f64", "f32"):
            fn = getattr(_lib, f"oracle_hdiff_{sfx}")
            fn.argtypes = [vp, vp, vp] + [i64] * 6
            fn.restype = ctypes.c_int
            fn = getattr(_lib, f"oracle_vadv_{sfx}")
            fn.argtypes = [vp] * 6 + [i64] * 8
            fn.restype = ctypes.c_int
        _lib.oracle_triad_f64.argtypes = [vp, vp, vp, ctypes.c_double, i64]
        _lib.oracle_triad_f64.restype = None
        _lib.oracle_max_threads.restype = ctypes.c_int
        _lib.oracle_set_threads.argtypes = [ctypes.c_int]
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def _interior_ptr(a, halo):
    off = int(np.sum(np.asarray(a.strides) * np.asarray(halo)))
    return a.ctypes.data + off


def _strides(a):
    return [s // a.itemsize for s in a.strides]


def _suffix(dtype):
    return {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}[np.dtype(dtype)]


def hdiff(inp, coeff, out, domain, halo):
    """out[interior] = hdiff(inp, coeff); arrays are halo'd, same strides."""
    assert inp.strides == coeff.strides == out.strides
    fn = getattr(lib(), f"oracle_hdiff_{_suffix(inp.dtype)}")
    rc = fn(_interior_ptr(inp, halo), _interior_ptr(coeff, halo), _interior_ptr(out, halo),
            *domain, *_strides(inp))
    if rc:
        raise MemoryError("oracle_hdiff failed to allocate its work planes")


def vadv(stage, pos, tens, tensstage, wcon, domain, halo, shift=(1, 0), out=None):
    """Thomas solve of one component; the new tensstage goes to ``out``
    (default: tensstage itself, the reference's in-place update)."""
    out = tensstage if out is None else out
    arrays = (stage, pos, tens, tensstage, wcon, out)
    assert all(a.strides == stage.strides for a in arrays)
    fn = getattr(lib(), f"oracle_vadv_{_suffix(stage.dtype)}")
    rc = fn(*[_interior_ptr(a, halo) for a in arrays], *domain, *_strides(stage), *shift)
    if rc == 2:
        raise ValueError("vertical advection needs at least 2 levels")
    if rc:
        raise MemoryError("oracle_vadv failed to allocate its work columns")


def triad(a, b, c, scalar):
    lib().oracle_triad_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, float(scalar), a.size)
