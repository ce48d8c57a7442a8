"""Continuous-batching server for hdiff / vadv solves on one GPU.

A request is one stencil solve (hdiff, or vadv u component) on its own domain
with a storage precision tag (float64, float32, or bfloat16 storage with
float32 compute).  Its fields live on the device from admission to
completion: the server allocates them from a budget-capped pool and creates
the inputs in place with the library's seeded generator (``sb_fill_batch``),
so request data never crosses the host link; the output stays on the device
for the client.

Scheduling (``Server.step``), repeated by the caller's loop:

1. poll: batches whose completion event has fired retire their requests
   (latency = completion seen - arrival) and return their memory to the pool;
2. admit: waiting requests, in arrival order, get their fields if the pool's
   budget allows (150 GB by default); one ``sb_fill_batch`` launch creates the
   inputs of everything admitted in this step;
3. dispatch: for every precision form with admitted requests and a free slot,
   up to ``max_batch`` of them are packed into that slot's ``Batch`` and
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

import collections
import ctypes
import math
import gc
import time
import weakref
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _native, kernels
from .batching import Batch, HdiffDomain, VadvDomain
from .device import DeviceBuffer, Event, Field, PinnedBuffer, Stream

ALIGN = 256  # field allocations start on 256-byte boundaries
FILL_DEPTH = 8  # page-locked staging slots for fill descriptors

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

    def domain(self):
        f = self.fields
        if self.op == "hdiff":
            return HdiffDomain(f["inp"], f["coeff"], f["out"])
        return VadvDomain(f["stage"], f["pos"], f["tens"], f["tensstage"], f["wcon"], out=f["out"])


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


def _event_done(event: Event) -> bool:
    rc = _native.lib().sb_event_query(ctypes.c_void_p(event.handle))
    if rc == _native.SB_NOT_READY:
        return False
    if rc != _native.SB_OK:
        raise _native.SbError("sb_event_query", rc, _native.last_error())
    return True


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


def _wait(stream: Stream, event: Event):
    _native.call("sb_stream_wait_event", stream.as_parameter, ctypes.c_void_p(event.handle))


@dataclass
class _Slot:
    batch: Batch
    stream: Stream
    done: Event
    requests: List[Request] = field(default_factory=list)
    busy: bool = False


class Server:
    def __init__(self, budget_bytes: float = 150e9, max_batch: int = 64, max_nk: int = 137, slots_per_form: int = 3,
                 keep_outputs: bool = False, batch_tune: Optional[dict] = None, fill_capacity: int = 4096,
                 float64_compute: str = "float64", mode: str = "batched", keep_inputs: bool = False):
        """``float64_compute`` picks how float64 requests are computed: "float64"
        (exact, bit-identical to the reference's numpy) or "fixed64" (fixed-point
        hdiff and float-pair vadv: errors within 1e-12 / 1e-10 of the field scale,
        about 3x less device time).  ``mode`` "batched" packs a slot's requests
        into one graph replay of the persistent kernels; "plain" launches each
        request's kernel on its own (the per-request baseline).  ``keep_outputs`` /
        ``keep_inputs`` keep a completed request's output / input fields until
        ``release``."""
        if float64_compute not in ("float64", "fixed64"):
            raise ValueError("float64_compute must be 'float64' or 'fixed64'")
        if mode not in ("batched", "plain"):
            raise ValueError("mode must be 'batched' or 'plain'")
        self.mode = mode
        _native.call("sb_set_device", 0)
        self.pool = DevicePool(int(budget_bytes))
        self.max_batch, self.max_nk = max_batch, max_nk
        self.keep_outputs = keep_outputs
        self.keep_inputs = keep_inputs
        self.float64_compute = float64_compute
        tune = dict(batch_tune or {})
        forms = dict(FORMS, float64=("float64", float64_compute))
        self.computes = {form: c for form, (_, c) in forms.items()}
        self.slots = {
            form: [_Slot(Batch(s, c, max_domains=max_batch, max_nk=max_nk, **tune) if mode == "batched" else None,
                         Stream(), Event())
                   for _ in range(slots_per_form)]
            for form, (s, c) in forms.items()
        }
        self.waiting: collections.deque = collections.deque()
        self.ready = {form: collections.deque() for form in FORMS}
        self.completed: List[Request] = []
        # fills go out on their own stream; their descriptors are staged in a
        # page-locked ring of FILL_DEPTH slots, each reused once the fill that
        # last read it has run (its event)
        self.fill_stream = Stream()
        self.fill_capacity = fill_capacity
        self.fill_scratch = DeviceBuffer(ctypes.sizeof(SbFillDesc) * fill_capacity)
        self.fill_staging = PinnedBuffer(ctypes.sizeof(SbFillDesc) * fill_capacity * FILL_DEPTH)
        self.fill_events = [Event() for _ in range(FILL_DEPTH)]
        self._fill_used = [False] * FILL_DEPTH
        self._fill_next = 0
        self.fill_done = self.fill_events[0]
        self.max_waiting = 0

    # -- client side ------------------------------------------------------------

    def submit(self, req: Request):
        if req.storage not in FORMS:
            raise ValueError(f"unknown precision {req.storage!r}")
        if req.op == "vadv" and req.nk > self.max_nk:
            raise ValueError(f"nk = {req.nk} exceeds the server's max_nk {self.max_nk}")
        if req.footprint() > self.pool.budget:
            raise ValueError("request larger than the whole memory budget")
        if req.arrival is None:
            req.arrival = time.perf_counter()
        self.waiting.append(req)
        self.max_waiting = max(self.max_waiting, len(self.waiting))

    def busy(self) -> bool:
        return bool(self.waiting) or any(self.ready.values()) or any(
            s.busy for slots in self.slots.values() for s in slots)

    def step(self):
        self._poll()
        self._admit()
        self._dispatch()

    def drain(self):
        while self.busy():
            self.step()

    def release(self, req: Request):
        """Return a completed request's kept fields to the pool."""
        for name in list(req.fields):
            self.pool.release(req.fields.pop(name).buffer)

    # -- scheduling -------------------------------------------------------------

    def _poll(self):
        for slots in self.slots.values():
            for slot in slots:
                if not slot.busy:
                    continue
                if not _event_done(slot.done):
                    continue
                now = time.perf_counter()
                for req in slot.requests:
                    req.completed = now
                    for name in list(req.fields):
                        if self.keep_outputs if name == "out" else self.keep_inputs:
                            continue
                        self.pool.release(req.fields.pop(name).buffer)
                    self.completed.append(req)
                slot.requests = []
                slot.busy = False

    def _admit(self):
        descs = []
        now = time.perf_counter()
        while self.waiting and len(descs) + 6 <= self.fill_capacity:
            req = self.waiting[0]
            specs = HDIFF_FIELDS if req.op == "hdiff" else VADV_FIELDS
            shape, strides, halo = field_layout(req.op, req.ni, req.nj, req.nk)
            count = math.prod(shape)
            bufs = []
            for _ in specs:
                buf = self.pool.try_alloc(count * ITEMSIZE[req.storage])
                if buf is None:
                    break
                bufs.append(buf)
            if len(bufs) < len(specs):  # budget exhausted: wait for completions (FIFO order kept)
                for buf in bufs:
                    self.pool.release(buf)
                break
            self.waiting.popleft()
            code = _native.storage_code(req.storage)
            for q, ((name, lo, hi), buf) in enumerate(zip(specs, bufs)):
                req.fields[name] = Field(buf, shape, strides, req.storage, halo)
                if lo is not None:
                    descs.append(SbFillDesc(buf.ptr, count, field_seed(req.seed, q), lo, hi, code, 0))
            req.admitted = now
            self.ready[req.storage].append(req)
        if descs:
            k = self._fill_next
            self._fill_next = (k + 1) % FILL_DEPTH
            if self._fill_used[k]:
                self.fill_events[k].synchronize()  # normally long done
            staging = self.fill_staging.ptr + k * self.fill_capacity * ctypes.sizeof(SbFillDesc)
            _fill(descs, self.fill_scratch, self.fill_stream, staging)
            self.fill_events[k].record(self.fill_stream)
            self._fill_used[k] = True
            self.fill_done = self.fill_events[k]

    def _dispatch(self):
        for form, queue in self.ready.items():
            while queue:
                slot = next((s for s in self.slots[form] if not s.busy), None)
                if slot is None:
                    break
                reqs = [queue.popleft() for _ in range(min(self.max_batch, len(queue)))]
                _wait(slot.stream, self.fill_done)
                if self.mode == "batched":
                    slot.batch.set([r.domain() for r in reqs])
                    slot.batch.launch(slot.stream)
                else:
                    for r in reqs:
                        self._launch_one(r, slot.stream)
                slot.done.record(slot.stream)
                now = time.perf_counter()
                for r in reqs:
                    r.launched = now
                slot.requests = reqs
                slot.busy = True


    def _launch_one(self, req: Request, stream: Stream):
        f = req.fields
        compute = self.computes[req.storage]
        if req.op == "hdiff":
            kernels.hdiff(f["inp"], f["coeff"], f["out"], compute=compute, stream=stream)
        else:
            kernels.vadv(f["stage"], f["pos"], f["tens"], f["tensstage"], f["wcon"], out=f["out"],
                         compute="float32x2" if compute == "fixed64" else compute, stream=stream)


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
    busy_host = 0.0  # time spent in Server.step with requests waiting or ready (host-side scheduling work)
    try:
        t0 = time.perf_counter()
        nxt = 0
        while nxt < len(requests) or server.busy():
            now = time.perf_counter() - t0
            while nxt < len(requests) and offsets[nxt] <= now:
                requests[nxt].arrival = t0 + offsets[nxt]
                server.submit(requests[nxt])
                nxt += 1
            pending = bool(server.waiting) or any(server.ready.values())
            s0 = time.perf_counter()
            server.step()
            if pending:
                busy_host += time.perf_counter() - s0
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
        "host_step_fraction": busy_host / (last - first),
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
