"""Continuous-batching server for hdiff / vadv solves on one GPU.

A request is one stencil solve (hdiff, or vadv u component) on its own domain
with a storage precision tag (float64, float32, or bfloat16 storage with
float32 compute).  Its fields live on the device from admission to
completion: the server allocates them from a budget-capped region and
creates the inputs in place with the library's seeded generator
(``sb_fill_batch``), so request data never crosses the host link; the output
stays on the device for the client.

The scheduler is native (``csrc/server.cu``, ``sb_server_*``); ``Server`` is
its Python face.  ``Server.step`` runs, in the library:

1. poll: batches whose completion event has fired retire their requests
   (latency = completion seen - arrival) and return their memory;
2. admit: waiting requests, in arrival order, get their fields if the
   budget allows (150 GB by default); one ``sb_fill_batch`` launch creates the
   inputs of everything admitted in this step;
3. dispatch: for every precision form with admitted requests and a free slot,
   up to ``max_batch`` of them are packed into that slot's batch and
   launched (one graph replay) on the slot's stream, after the fill.

Several slots per form are in flight at once, so requests that arrive while
others run are admitted as memory frees up and their work overlaps on the
device (continuous batching, not a queue in front of one launch at a time).
Every result is computed by the same per-item arithmetic wherever and with
whatever it is batched, so it is bit-identical alone and in a mix.

``Server(mode="plain")`` is the comparison without batching: the same
admission, fill, slots and streams, but every request is its own
``sb_hdiff`` / ``sb_vadv`` launch (the library's default form for its size
and precision) instead of a place in a batched graph replay.

``run_load`` drives a server with a Poisson arrival process in real time.
"""

from __future__ import annotations

import ctypes
import gc
import itertools
import math
import time
import weakref
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _native
from .batching import SbBatchTune
from .device import DeviceBuffer, Field, Stream

ALIGN = 256  # field allocations start on 256-byte boundaries

FORMS = {"float64": ("float64", "float64"), "float32": ("float32", "float32"), "bfloat16": ("bfloat16", "float32")}
ITEMSIZE = {"float64": 8, "float32": 4, "bfloat16": 2}

HDIFF_FIELDS = (("inp", 0.0, 1.0), ("coeff", 0.0, 1.0), ("out", None, None))
VADV_FIELDS = (("stage", -1.0, 1.0), ("pos", -1.0, 1.0), ("tens", -1.0, 1.0), ("tensstage", -1.0, 1.0),
               ("wcon", -0.5, 0.5), ("out", None, None))
HALO = {"hdiff": (2, 2, 0), "vadv": (1, 1, 0)}


class SbFillDesc(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("count", ctypes.c_int64), ("seed", ctypes.c_uint64),
                ("lo", ctypes.c_double), ("hi", ctypes.c_double), ("storage", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


def field_seed(request_seed: int, index: int) -> int:
    """Seed of field ``index`` of a request (a fixed mix of the request seed)."""
    return (request_seed * 0x9E3779B97F4A7C15 + (index + 1) * 0xD1B54A32D192ED03) % (1 << 64)


def field_layout(op: str, ni: int, nj: int, nk: int):
    """(shape, element strides, halo) of a request field: i unit-stride, no padding."""
    hi, hj, hk = HALO[op]
    shape = (ni + 2 * hi, nj + 2 * hj, nk + 2 * hk)
    return shape, (1, shape[0], shape[0] * shape[1]), HALO[op]


@dataclass
class Request:
    rid: int
    op: str  # "hdiff" or "vadv"
    ni: int
    nj: int
    nk: int
    storage: str  # "float64", "float32" or "bfloat16"
    seed: int
    arrival: Optional[float] = None
    admitted: Optional[float] = None
    launched: Optional[float] = None
    completed: Optional[float] = None
    fields: Dict[str, Field] = field(default_factory=dict)

    @property
    def points(self) -> int:
        return self.ni * self.nj * self.nk

    @property
    def latency(self) -> float:
        return self.completed - self.arrival

    def footprint(self) -> int:
        shape, _, _ = field_layout(self.op, self.ni, self.nj, self.nk)
        n = len(HDIFF_FIELDS if self.op == "hdiff" else VADV_FIELDS)
        return n * _round(math.prod(shape) * ITEMSIZE[self.storage])



def _round(nbytes: int) -> int:
    return max(ALIGN, -(-nbytes // ALIGN) * ALIGN)


@dataclass
class Block:
    """A piece of the pool's device region (what a Field needs of a buffer)."""

    ptr: int
    nbytes: int


class DevicePool:
    """Budget-capped device memory: the whole budget is allocated once and
    carved by the library's best-fit arena (``sb_arena_*``), so admitting and
    retiring requests makes no CUDA allocation call (cudaMalloc / cudaFree
    synchronise the device and would stall every batch in flight)."""

    def __init__(self, budget_bytes: int):
        self.budget = int(budget_bytes) // ALIGN * ALIGN
        self.region = DeviceBuffer(self.budget)
        self._lib = _native.lib()
        handle = ctypes.c_void_p()
        self._check("sb_arena_create", self._lib.sb_arena_create(ctypes.byref(handle), self.region.ptr,
                                                                 self.budget, ALIGN))
        self._arena = handle.value
        self._finalizer = weakref.finalize(self, self._lib.sb_arena_destroy, ctypes.c_void_p(self._arena))

    @staticmethod
    def _check(name, rc):
        if rc != _native.SB_OK:
            raise _native.SbError(name, rc, _native.last_error())

    def try_alloc(self, nbytes: int) -> Optional[Block]:
        """A block of at least ``nbytes`` bytes, or None when no free piece is large enough."""
        addr = ctypes.c_uint64()
        rc = self._lib.sb_arena_alloc(ctypes.c_void_p(self._arena), max(1, int(nbytes)), ctypes.byref(addr))
        if rc == _native.SB_ERR_BUDGET:
            return None
        self._check("sb_arena_alloc", rc)
        return Block(addr.value, _round(nbytes))

    def release(self, block: Block):
        self._check("sb_arena_free", self._lib.sb_arena_free(ctypes.c_void_p(self._arena), block.ptr))

    def stats(self) -> Dict[str, int]:
        vals = [ctypes.c_uint64() for _ in range(4)]
        self._check("sb_arena_stats", self._lib.sb_arena_stats(ctypes.c_void_p(self._arena),
                                                               *[ctypes.byref(v) for v in vals]))
        return dict(zip(("in_use", "peak", "largest_free", "free_blocks"), (v.value for v in vals)))

    @property
    def in_use(self) -> int:
        return self.stats()["in_use"]

    @property
    def peak(self) -> int:
        return self.stats()["peak"]


def _fill(descs, scratch: DeviceBuffer, stream: Stream, staging: Optional[int] = None):
    """Generate the fields ``descs`` describe on ``stream``.  With ``staging``
    (page-locked host memory for ``len(descs)`` descriptors, left untouched
    until the stream has run the fill) the descriptor copy is queued; from
    pageable memory it first waits for ``stream`` to drain."""
    arr = (SbFillDesc * len(descs))(*descs)
    src = ctypes.addressof(arr)
    if staging is not None:
        ctypes.memmove(staging, src, ctypes.sizeof(arr))
        src = staging
    _native.call("sb_fill_batch", ctypes.c_void_p(src), len(descs), ctypes.c_void_p(scratch.ptr), stream.as_parameter)


class SbServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_int32), ("max_nk", ctypes.c_int32),
                ("slots_per_form", ctypes.c_int32), ("float64_compute", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("keep", ctypes.c_int32), ("fill_capacity", ctypes.c_int32), ("simulate", ctypes.c_int32),
                ("tune", SbBatchTune)]


class SbRequest(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("op", ctypes.c_int32), ("storage", ctypes.c_int32), ("ni", ctypes.c_int64),
                ("nj", ctypes.c_int64), ("nk", ctypes.c_int64), ("seed", ctypes.c_uint64), ("arrival", ctypes.c_double)]


class SbCompletion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("arrival", ctypes.c_double), ("admitted", ctypes.c_double),
                ("launched", ctypes.c_double), ("completed", ctypes.c_double)]


class SbServerState(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("in_use_bytes", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("waiting", ctypes.c_int64), ("ready", ctypes.c_int64), ("inflight", ctypes.c_int64),
                ("max_waiting", ctypes.c_int64), ("busy_slots", ctypes.c_int64), ("work_seconds", ctypes.c_double)]


class SbServerLaunch(ctypes.Structure):
    _fields_ = [("storage", ctypes.c_int32), ("requests", ctypes.c_int32)]


_STORAGE_NAME = {_native.DTYPE_CODES[f]: f for f in FORMS}


class _PoolView:
    """Memory counters of a server's region (bytes)."""

    def __init__(self, server):
        self._server = server

    @property
    def budget(self) -> int:
        return self._server.state().budget_bytes

    @property
    def in_use(self) -> int:
        return self._server.state().in_use_bytes

    @property
    def peak(self) -> int:
        return self._server.state().peak_bytes


class Server:
    """The native continuous-batching server (sb_server_*), driven from Python.

    Per request Python makes one call (``submit``); ``step`` runs the native
    poll / admit / dispatch and hands back the completed requests.  The
    Request objects given to ``submit`` get their ``admitted`` /
    ``launched`` / ``completed`` times (on ``time.perf_counter``'s clock) when
    they complete, and their kept fields (``keep_outputs`` / ``keep_inputs``)
    as ``Field`` objects in ``fields`` until ``release``."""

    def __init__(self, budget_bytes: float = 150e9, max_batch: int = 64, max_nk: int = 137, slots_per_form: int = 3,
                 keep_outputs: bool = False, batch_tune: Optional[dict] = None, fill_capacity: int = 4096,
                 float64_compute: str = "float64", mode: str = "batched", keep_inputs: bool = False,
                 simulate: bool = False):
        """``float64_compute`` picks how float64 requests are computed: "float64"
        (exact, bit-identical to the reference's numpy) or "fixed64" (fixed-point
        hdiff, 4e-16 of the field scale, and float-pair vadv, about 48
        significant bits, within 1e-10 of the field scale except in
        near-singular columns; about 3x less device time).  ``mode`` "batched" packs a slot's requests
        into one graph replay of the persistent kernels; "plain" launches each
        request's kernel on its own (the per-request baseline).  ``simulate``
        runs the scheduling without any device work (tests)."""
        if float64_compute not in ("float64", "fixed64"):
            raise ValueError("float64_compute must be 'float64' or 'fixed64'")
        if mode not in ("batched", "plain"):
            raise ValueError("mode must be 'batched' or 'plain'")
        self.mode = mode
        self.max_nk = max_nk
        self._lib = _native.lib()
        cfg = SbServerConfig(budget_bytes=int(budget_bytes), max_batch=max_batch, max_nk=max_nk,
                             slots_per_form=slots_per_form,
                             float64_compute=_native.DTYPE_CODES["fixed64" if float64_compute == "fixed64" else "float64"],
                             mode=0 if mode == "batched" else 1, keep=(1 if keep_outputs else 0) | (2 if keep_inputs else 0),
                             fill_capacity=fill_capacity, simulate=1 if simulate else 0)
        for k, v in (batch_tune or {}).items():
            setattr(cfg.tune, k, int(v))
        handle = ctypes.c_void_p()
        self._check("sb_server_create", self._lib.sb_server_create(ctypes.byref(handle), ctypes.byref(cfg)))
        self._handle = handle
        self._finalizer = weakref.finalize(self, self._lib.sb_server_destroy, handle)
        self.completed: List[Request] = []
        self._held: Dict[int, Request] = {}
        self._ids = itertools.count()
        self._done = (SbCompletion * 1024)()
        self._busy = ctypes.c_int(0)
        self._req = SbRequest()

    @staticmethod
    def _check(name, rc):
        if rc != _native.SB_OK:
            raise _native.SbError(name, rc, _native.last_error())

    @property
    def pool(self) -> _PoolView:
        return _PoolView(self)

    def close(self):
        """Wait for the device work and free the server's region now."""
        self._finalizer()

    # -- client side ------------------------------------------------------------

    def submit(self, req: Request):
        if req.storage not in FORMS:
            raise ValueError(f"unknown precision {req.storage!r}")
        if req.arrival is None:
            req.arrival = time.perf_counter()
        key = next(self._ids)
        r = self._req
        r.id, r.op, r.storage = key, 0 if req.op == "hdiff" else 1, _native.DTYPE_CODES[req.storage]
        r.ni, r.nj, r.nk, r.seed, r.arrival = req.ni, req.nj, req.nk, req.seed % (1 << 64), req.arrival
        rc = self._lib.sb_server_submit(self._handle, ctypes.byref(r))
        if rc == _native.SB_ERR_INVALID:
            raise ValueError(_native.last_error())
        self._check("sb_server_submit", rc)
        req._key = key
        self._held[key] = req

    def step(self, now: Optional[float] = None) -> bool:
        """One poll / admit / dispatch; True while requests are waiting, queued
        or on the device."""
        self._check("sb_server_step", self._lib.sb_server_step(self._handle, ctypes.c_double(
            time.perf_counter() if now is None else now), ctypes.byref(self._busy)))
        self._collect()
        return bool(self._busy.value)

    def busy(self) -> bool:
        st = self.state()
        return bool(st.waiting or st.ready or st.inflight)

    def drain(self):
        while self.step():
            pass

    def release(self, req: Request):
        """Return a completed request's kept fields to the pool."""
        if req.fields:
            self._check("sb_server_release", self._lib.sb_server_release(self._handle, ctypes.c_int64(req._key)))
        req.fields.clear()

    def query(self, req: Request) -> Request:
        """Refresh the times of a request the server still holds."""
        rec = SbCompletion()
        if self._lib.sb_server_query(self._handle, ctypes.c_int64(req._key), ctypes.byref(rec)) == _native.SB_OK:
            req.admitted, req.launched, req.completed = (v if v >= 0.0 else None
                                                         for v in (rec.admitted, rec.launched, rec.completed))
        return req

    def state(self) -> SbServerState:
        st = SbServerState()
        self._check("sb_server_stats", self._lib.sb_server_stats(self._handle, ctypes.byref(st)))
        return st

    @property
    def max_waiting(self) -> int:
        return self.state().max_waiting

    def debug_complete(self):
        """Simulating server: finish every batch in flight."""
        self._check("sb_server_debug_complete", self._lib.sb_server_debug_complete(self._handle))

    def launches(self):
        """Simulating server: the launches so far, as (storage, requests)."""
        n = ctypes.c_int(0)
        self._lib.sb_server_debug_launches(self._handle, None, 0, ctypes.byref(n))
        out = (SbServerLaunch * max(1, n.value))()
        self._check("sb_server_debug_launches",
                    self._lib.sb_server_debug_launches(self._handle, out, n.value, ctypes.byref(n)))
        return [(_STORAGE_NAME[out[q].storage], out[q].requests) for q in range(n.value)]

    # -- completions --------------------------------------------------------------

    def _collect(self):
        n = ctypes.c_int(0)
        while True:
            self._check("sb_server_take_completed",
                        self._lib.sb_server_take_completed(self._handle, self._done, len(self._done), ctypes.byref(n)))
            for q in range(n.value):
                rec = self._done[q]
                req = self._held.pop(rec.id)
                req.admitted, req.launched, req.completed = rec.admitted, rec.launched, rec.completed
                self._attach_kept(req)
                self.completed.append(req)
            if n.value < len(self._done):
                return

    def _attach_kept(self, req: Request):
        specs = HDIFF_FIELDS if req.op == "hdiff" else VADV_FIELDS
        shape, strides, halo = field_layout(req.op, req.ni, req.nj, req.nk)
        nbytes = math.prod(shape) * ITEMSIZE[req.storage]
        ptr = ctypes.c_void_p()
        for q, (name, _, _) in enumerate(specs):
            if self._lib.sb_server_field(self._handle, ctypes.c_int64(req._key), q, ctypes.byref(ptr)) == _native.SB_OK:
                req.fields[name] = Field(Block(ptr.value, nbytes), shape, strides, req.storage, halo)


# ---------------------------------------------------------------------------
# workload and load driver
# ---------------------------------------------------------------------------


def request_specs(n: int, seed: int = 11, sizes=(32, 1024), nk=(40, 137), mix=(0.2, 0.6, 0.2)):
    """Requests of the serving workload: op 50/50, ni and nj log-uniform in
    ``sizes`` rounded to a multiple of 32, nk uniform in ``nk`` (inclusive),
    precision float64 / float32 / bfloat16 with probabilities ``mix``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi = math.log(sizes[0]), math.log(sizes[1])
    forms = ("float64", "float32", "bfloat16")
    reqs = []
    for rid in range(n):
        op = "hdiff" if rng.random() < 0.5 else "vadv"
        ni, nj = (max(32, int(round(math.exp(rng.uniform(lo, hi)) / 32.0)) * 32) for _ in range(2))
        k = int(rng.integers(nk[0], nk[1] + 1))
        storage = forms[int(rng.choice(3, p=mix))]
        reqs.append(Request(rid, op, ni, nj, k, storage, int(rng.integers(0, 2**62))))
    return reqs


def run_load(server: Server, requests: List[Request], rate: float, seed: int = 5):
    """Submit ``requests`` with Poisson arrivals at ``rate`` per second (in real
    time) and step the server until all complete.  Returns summary statistics."""
    rng = np.random.Generator(np.random.PCG64(seed))
    offsets = np.cumsum(rng.exponential(1.0 / rate, size=len(requests)))
    # no cyclic-garbage pauses inside the latency-critical loop (collected once before)
    gc.collect()
    gc_was_enabled = gc.isenabled()
    gc.disable()
    work0 = server.state().work_seconds
    try:
        t0 = time.perf_counter()
        nxt = 0
        busy = True
        while nxt < len(requests) or busy:
            now = time.perf_counter() - t0
            while nxt < len(requests) and offsets[nxt] <= now:
                requests[nxt].arrival = t0 + offsets[nxt]
                server.submit(requests[nxt])
                nxt += 1
            busy = server.step()
    finally:
        if gc_was_enabled:
            gc.enable()
    lat = np.array([r.latency for r in requests])
    first = min(r.arrival for r in requests)
    last = max(r.completed for r in requests)
    points = sum(r.points for r in requests)
    by_form = {}
    for form in FORMS:
        fl = [r.latency for r in requests if r.storage == form]
        if fl:
            by_form[form] = {"n": len(fl), "p50_ms": float(np.percentile(fl, 50) * 1e3),
                             "p99_ms": float(np.percentile(fl, 99) * 1e3)}
    return {
        "rate_offered": rate,
        "requests": len(requests),
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "mean_ms": float(lat.mean() * 1e3),
        "throughput_req_s": len(requests) / (last - first),
        "gpoints_s": points / (last - first) / 1e9,
        "peak_pool_gb": server.pool.peak / 1e9,
        "max_waiting": server.max_waiting,
        "host_step_fraction": (server.state().work_seconds - work0) / (last - first),
        "by_precision": by_form,
    }


def main(argv=None):
    """Sweep Poisson arrival rates over the serving workload; one JSON line per rate."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description="continuous-batching serving sweep")
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--rates", default="1000,2000,5000,10000,20000,50000")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--float64-compute", choices=["float64", "fixed64"], default="float64",
                    help="float64 requests: exact (float64) or fixed-point hdiff / float-pair vadv (fixed64)")
    ap.add_argument("--mode", choices=["batched", "plain"], default="batched",
                    help="batched graph replays, or one kernel launch per request")
    args = ap.parse_args(argv)
    server = Server(budget_bytes=args.budget_gb * 1e9, max_batch=args.max_batch, slots_per_form=args.slots,
                    float64_compute=args.float64_compute, mode=args.mode)
    warm = request_specs(1024, seed=args.seed + 1000)  # every slot launches (and captures its graph) once
    run_load(server, warm, rate=1e6)
    for rate in (float(r) for r in args.rates.split(",")):
        reqs = request_specs(args.requests, seed=args.seed)
        print(json.dumps(run_load(server, reqs, rate=rate)), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
