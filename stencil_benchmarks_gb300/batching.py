"""Batched execution of many hdiff / vadv domains in one persistent launch.

``Batch`` wraps ``sb_batch_*``: a fixed-capacity domain table, device-side
work queues and a CUDA graph (table upload -> queue reset -> persistent hdiff
kernel side by side with one persistent vadv kernel per nk bucket) that
``launch()`` replays.  Every domain
of a batch has the same storage/compute form.  Results are bit-identical to
launching ``kernels.hdiff`` / ``kernels.vadv`` on each domain.

    batch = Batch("float32", max_domains=64, max_nk=137)
    batch.set([HdiffDomain(inp, coeff, out), VadvDomain(stage, pos, tens, tensstage, wcon), ...])
    seconds = batch.launch(timed=True)
"""

from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass
from typing import Optional, Sequence, Union

from . import _native
from .device import Field, _stream_arg

SB_OP_HDIFF, SB_OP_VADV = 0, 1


class SbDomain(ctypes.Structure):
    _fields_ = [
        ("op", ctypes.c_int32),
        ("wshift_i", ctypes.c_int32),
        ("wshift_j", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("ni", ctypes.c_int64), ("nj", ctypes.c_int64), ("nk", ctypes.c_int64),
        ("si", ctypes.c_int64), ("sj", ctypes.c_int64), ("sk", ctypes.c_int64),
        ("f", ctypes.c_void_p * 5),
        ("out", ctypes.c_void_p),
    ]


class SbBatchTune(ctypes.Structure):
    _fields_ = [
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("hdiff_rows", ctypes.c_int32),
        ("hdiff_planes", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("vadv_block", ctypes.c_int32),
        ("vadv_blocks_per_sm", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


@dataclass
class HdiffDomain:
    inp: Field
    coeff: Field
    out: Field


@dataclass
class VadvDomain:
    stage: Field
    pos: Field
    tens: Field
    tensstage: Field
    wcon: Field
    out: Optional[Field] = None  # default: tensstage (in place)
    shift: tuple = (1, 0)


Domain = Union[HdiffDomain, VadvDomain]


def _interior(field: Field):
    return tuple(n - 2 * h for n, h in zip(field.shape, field.halo))


def to_sb_domain(d: Domain) -> SbDomain:
    s = SbDomain()
    if isinstance(d, HdiffDomain):
        fields = [d.inp, d.coeff]
        out = d.out
        s.op = SB_OP_HDIFF
        if min(d.inp.halo[:2]) < 2:
            raise ValueError("horizontal diffusion needs a halo of at least 2 in i and j")
    else:
        fields = [d.stage, d.pos, d.tens, d.tensstage, d.wcon]
        out = d.out if d.out is not None else d.tensstage
        s.op = SB_OP_VADV
        s.wshift_i, s.wshift_j = d.shift
        if any(h < sh for h, sh in zip(d.stage.halo[:2], d.shift)):
            raise ValueError("vertical advection needs a halo >= 1 along the wcon shift")
    base = fields[0]
    for f in fields + [out]:
        if f.strides != base.strides or f.shape != base.shape or f.storage != base.storage:
            raise ValueError("all fields of a domain must share shape, strides and storage type")
    s.ni, s.nj, s.nk = _interior(base)
    s.si, s.sj, s.sk = base.strides
    for q, f in enumerate(fields):
        s.f[q] = f.interior_ptr
    s.out = out.interior_ptr
    return s


def _sigs():
    lib = _native.lib()
    if getattr(lib, "_sb_batch_ready", False):
        return lib
    vp, i64 = ctypes.c_void_p, ctypes.c_int64
    lib.sb_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, i64,
                                    ctypes.POINTER(SbBatchTune)]
    lib.sb_batch_set.argtypes = [vp, ctypes.POINTER(SbDomain), ctypes.c_int]
    lib.sb_batch_launch.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_double)]
    lib.sb_batch_info.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_size_t),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.sb_batch_destroy.argtypes = [vp]
    for name in ("sb_batch_create", "sb_batch_set", "sb_batch_launch", "sb_batch_info", "sb_batch_destroy"):
        getattr(lib, name).restype = ctypes.c_int
    lib._sb_batch_ready = True
    return lib


class Batch:
    """A reusable batch of up to ``max_domains`` domains of one form."""

    def __init__(self, storage: str, compute: Optional[str] = None, max_domains: int = 64, max_nk: int = 256,
                 block: int = 0, blocks_per_sm: int = 0, hdiff_rows: int = 0, hdiff_planes: int = 0,
                 order: int = 0, vadv_block: int = 0, vadv_blocks_per_sm: int = 0):
        lib = _sigs()
        compute = compute or ("float64" if storage == "float64" else "float32")
        self.storage, self.compute = storage, compute
        self.max_domains, self.max_nk = max_domains, max_nk
        tune = SbBatchTune(block=block, blocks_per_sm=blocks_per_sm, hdiff_rows=hdiff_rows,
                           hdiff_planes=hdiff_planes, order=order, vadv_block=vadv_block,
                           vadv_blocks_per_sm=vadv_blocks_per_sm)
        handle = ctypes.c_void_p()
        rc = lib.sb_batch_create(ctypes.byref(handle), _native.storage_code(storage), _native.storage_code(compute),
                                 int(max_domains), int(max_nk), ctypes.byref(tune))
        if rc:
            raise _native.SbError("sb_batch_create", rc, _native.last_error())
        self.handle = handle.value
        self._finalizer = weakref.finalize(self, Batch._release, self.handle)
        self._domains: Sequence[Domain] = ()

    @staticmethod
    def _release(handle):
        try:
            _native.lib().sb_batch_destroy(ctypes.c_void_p(handle))
        except Exception:  # noqa: BLE001
            pass

    def close(self):
        self._finalizer()

    def set(self, domains: Sequence[Domain]):
        """Install a new set of domains (wait for earlier launches of this batch first)."""
        arr = (SbDomain * max(1, len(domains)))(*[to_sb_domain(d) for d in domains])
        rc = _sigs().sb_batch_set(ctypes.c_void_p(self.handle), arr, len(domains))
        if rc:
            raise _native.SbError("sb_batch_set", rc, _native.last_error())
        self._domains = list(domains)

    def launch(self, stream=None, timed: bool = False):
        t = ctypes.c_double(0.0)
        rc = _sigs().sb_batch_launch(ctypes.c_void_p(self.handle), _stream_arg(stream),
                                     ctypes.byref(t) if timed else None)
        if rc:
            raise _native.SbError("sb_batch_launch", rc, _native.last_error())
        return t.value if timed else None

    def info(self) -> dict:
        items, ws = ctypes.c_int64(), ctypes.c_size_t()
        grid, block = ctypes.c_int(), ctypes.c_int()
        rc = _sigs().sb_batch_info(ctypes.c_void_p(self.handle), ctypes.byref(items), ctypes.byref(ws),
                                   ctypes.byref(grid), ctypes.byref(block))
        if rc:
            raise _native.SbError("sb_batch_info", rc, _native.last_error())
        return {"items": items.value, "workspace_bytes": ws.value, "grid": grid.value, "block": block.value}
