"""Benchmark of the GB300 stencil backend on the 512x512x80 fp64 roofline set.

One step = one horizontal-diffusion launch (inp, coeff -> out) followed by
one vertical-advection launch (u component, in place), both on the interior
512 x 512 x 80 in fp64, with the reference's halos (2 in i/j for hdiff, 1 in
i for vadv) and seeded inputs drawn from the distributions of the workload
(hdiff fields U[0,1); vadv stage/pos/tens/tensstage U[-1,1), wcon
U[-0.5,0.5)).  The fields of one step occupy ~1.35 GB, far above the 129 MB
L2, so no L2 flush is needed between steps.

Printed JSON line (rank 0):
  value        grid points per second over the whole job (hdiff + vadv points,
               i.e. 2 * 512*512*80 per step per GPU), inputs resident in HBM
  e2e          the same metric through the C ABI with pinned host buffers:
               every step uploads the step's inputs and downloads its outputs
  roofline     the dominant kernel's compulsory HBM bytes per launch / its
               average CUDA-event duration, against the measured copy peak
  cpu_baseline the C restatement of the reference arithmetic (OpenMP, all
               host cores) on the same workload; `reference_backends` beside
               it times the reference's own OpenMP hdiff/vadv classes and its
               numpy hdiff through its Benchmark API
  stream_triad STREAM triad on 2^29 fp64 (the bandwidth calibration kernel)
  fast_f64     the same step with fixed-point hdiff and float-pair vadv
               (within the stated tolerances, not bit-identical), with its
               error against the exact step's outputs

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU (torchrun, one rank per GPU): every rank runs an independent
replica of the workload (weak scaling); ranks meet at a barrier around the
timed region and the maximum time over ranks is reported.
"""

from __future__ import annotations

import argparse
import contextlib
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NI, NJ, NK = 512, 512, 80
HDIFF_HALO = (2, 2, 0)
VADV_HALO = (1, 1, 0)
POINTS = NI * NJ * NK
TRIAD_N = 1 << 29
METRIC = "hdiff+vadv GPoints/s (fp64, 512x512x80)"
UNIT = "GPoints/s"
# the workload, identical in both arms' lines
CONFIG = {"workload": "hdiff+vadv fp64 512x512x80 (halo 2,2,0 / 1,1,0)",
          "l2": "inputs > L2 (1.35 GB of fields per step), no flush"}
# timed repetitions of the pipelined end-to-end loop (median reported)
E2E_REPS = 3


# fp64 vadv on GB300 is bound by the fp64 pipe; the SLAB variant (persistent
# threads, factors in compact slabs of the ccol/dcol scratch fields) keeps the
# most columns in flight and is the fastest exact form.  Its nine products and
# its pivot reciprocal per level run as integer arithmetic (bit-identical),
# which needs many blocks per SM to hide the longer integer sequences: a ring
# of depth 1, the library's 28 blocks per SM balanced to 27 (k_per_cta 0):
# about 740 us against 1175 us all-fp64.
VADV_TUNE = {"variant": 3, "block_x": 32, "unroll": 1, "k_per_cta": 0}

# The fast float64 step: hdiff with exact 64-bit fixed-point sums and one
# float64 FMA per point (float64 rounding level), vadv in float-pair
# arithmetic on the fp32 pipe (~48-bit significand; within 1e-10 of the
# field scale).  Neither is bit-identical to the reference's numpy.
FAST_HDIFF_COMPUTE = "fixed64"
FAST_VADV_COMPUTE = "float32x2"
FAST_VADV_TUNE = {"variant": 3, "block_x": 64, "unroll": 2, "k_per_cta": 32}


# Algorithmic fp64 operations per grid point of the reference's arithmetic
# (the exact kernels' ceiling on GB300): hdiff about 16 (Laplacian once per
# point, two limited fluxes, the update); vadv about 26 plus one divide.
FP64_OPS = {"hdiff": 16, "vadv": 27}


def compulsory_bytes(kind, s=8):
    """Algorithmic HBM bytes per launch (each input read once, output written once)."""
    if kind == "hdiff":  # inp with its 2-point i/j halo, coeff, out
        return s * ((NI + 4) * (NJ + 4) * NK + 2 * NI * NJ * NK)
    if kind == "vadv":  # ustage, upos, utens, utensstage (read + write), wcon incl. column i+1
        return s * (5 * NI * NJ * NK + (NI + 1) * NJ * NK)
    raise ValueError(kind)


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            data = json.loads(path.read_text())
            return float(data["hbm_gbs"]), "measured"
        except Exception:  # noqa: BLE001
            pass
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes from the committed ncu summary, if present."""
    path = ROOT / "profiles" / "dram_traffic.txt"
    out = {}
    if path.exists():
        for line in path.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.device_index = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power = [], [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None, "samples": len(sm),
                "reasons": sorted(reasons)}


class GpuUtilSampler(ClockSampler):
    """Mean nvidia-smi utilization.gpu (percent of time a kernel was running)
    over a window."""

    QUERY = "index,utilization.gpu"

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        vals = []
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            try:
                vals.append(float(parts[1]))
            except (IndexError, ValueError):
                continue
        return statistics.mean(vals) if vals else None


# ---------------------------------------------------------------------------
# distributed plumbing (torchrun): barrier and max over ranks
# ---------------------------------------------------------------------------


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend)
            self.torch, self.dist = torch, dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, value: float) -> float:
        if self.world == 1:
            return value
        dev = "cuda" if self.torch.cuda.is_available() else "cpu"
        t = self.torch.tensor([value], dtype=self.torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------


def make_inputs(seed=2024):
    from stencil_benchmarks_gb300 import array as sbarray

    rng = np.random.Generator(np.random.PCG64(seed))

    def field(halo, lo, hi):
        shape = (NI + 2 * halo[0], NJ + 2 * halo[1], NK + 2 * halo[2])
        a = sbarray.alloc_array(shape, "float64", (2, 1, 0), 0, index_to_align=halo)
        a[...] = rng.uniform(lo, hi, size=shape)
        return a

    hd = {n: field(HDIFF_HALO, 0.0, 1.0) for n in ("inp", "coeff", "out")}
    hd["out_fast"] = field(HDIFF_HALO, 0.0, 0.0)
    va = {n: field(VADV_HALO, -1.0, 1.0) for n in ("ustage", "upos", "utens", "utensstage")}
    va["wcon"] = field(VADV_HALO, -0.5, 0.5)
    # the new utensstage goes to a separate field, so every step solves the same system
    va["out"] = field(VADV_HALO, 0.0, 0.0)
    va["out_fast"] = field(VADV_HALO, 0.0, 0.0)
    # the reference's ccol/dcol fields: scratch for the forward-elimination factors
    va["ccol"] = field(VADV_HALO, 0.0, 0.0)
    va["dcol"] = field(VADV_HALO, 0.0, 0.0)
    return hd, va


def run_gpu(args, dist):
    from stencil_benchmarks_gb300 import _native, kernels
    from stencil_benchmarks_gb300.device import DeviceBuffer, Event, Field, PinnedBuffer, Stream

    _native.call("sb_set_device", dist.local_rank)
    info = _native.device_info(dist.local_rank)
    hd, va = make_inputs(seed=2024 + dist.rank)
    dev_hd = {n: Field.like_host(h, "float64", HDIFF_HALO) for n, h in hd.items()}
    dev_va = {n: Field.like_host(h, "float64", VADV_HALO) for n, h in va.items()}
    for n, h in hd.items():
        dev_hd[n].upload(h)
    for n, h in va.items():
        dev_va[n].upload(h)
    stream = Stream()
    launches = {"hdiff": 0, "vadv": 0}

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        kernels.hdiff(dev_hd["inp"], dev_hd["coeff"], dev_hd["out"], stream=stream)
        if ev is not None:
            ev[1].record(stream)
        kernels.vadv(dev_va["ustage"], dev_va["upos"], dev_va["utens"], dev_va["utensstage"], dev_va["wcon"],
                     out=dev_va["out"], ccol=dev_va["ccol"], dcol=dev_va["dcol"], tune=VADV_TUNE, stream=stream)
        if ev is not None:
            ev[2].record(stream)
        launches["hdiff"] += 1
        launches["vadv"] += 1

    for _ in range(args.warmup):
        step()
    stream.synchronize()

    events = [[Event(), Event(), Event()] for _ in range(args.steps)]
    start, stop = Event(), Event()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    time.sleep(0.3)
    dist.barrier()
    _native.synchronize()
    launches = {"hdiff": 0, "vadv": 0}
    start.record(stream)
    for s in range(args.steps):
        step(events[s])
    stop.record(stream)
    stop.synchronize()
    _native.synchronize()
    elapsed = start.elapsed(stop)
    dist.barrier()
    clk = clocks.stop()
    t_hdiff = [e[0].elapsed(e[1]) for e in events]
    t_vadv = [e[1].elapsed(e[2]) for e in events]
    elapsed_max = dist.max(elapsed)
    gpu_launches = launches["hdiff"] + launches["vadv"]

    # ---- end to end: pinned host buffers, H2D of the step's inputs, D2H of its outputs
    # inputs of a step: hdiff inp/coeff and the five vadv inputs (ccol/dcol are scratch)
    in_fields = [(dev_hd[n], hd[n]) for n in ("inp", "coeff")] + \
                [(dev_va[n], va[n]) for n in ("ustage", "upos", "utens", "utensstage", "wcon")]
    out_fields = [(dev_hd["out"], hd["out"]), (dev_va["out"], va["out"])]
    pinned_in = []
    for f, h in in_fields:
        pb = PinnedBuffer(f.span_bytes)
        view = pb.array(np.uint8, (f.span_bytes,))
        from stencil_benchmarks_gb300.device import _span_view

        view[...] = _span_view(h)
        pinned_in.append((f, pb))
    pinned_out = [(f, PinnedBuffer(f.span_bytes)) for f, _ in out_fields]
    h2d = sum(f.span_bytes for f, _ in pinned_in)
    d2h = sum(f.span_bytes for f, _ in pinned_out)

    def e2e_step():
        for f, pb in pinned_in:
            _native.call("sb_memcpy_async", f.base_ptr, pb.ptr, f.span_bytes, _native.H2D, stream.as_parameter)
        step()
        for f, pb in pinned_out:
            _native.call("sb_memcpy_async", pb.ptr, f.base_ptr, f.span_bytes, _native.D2H, stream.as_parameter)

    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(2):
        e2e_step()
    stream.synchronize()
    dist.barrier()
    e0, e1 = Event(), Event()
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    e1.synchronize()
    e2e_serial_time = dist.max(e0.elapsed(e1))

    # ---- end to end, pipelined: two device sets, uploads / compute / downloads
    # on their own streams, so step n+1's uploads and step n-1's downloads overlap
    # step n's kernels (every step still moves its own inputs and outputs)
    second = ({n: Field.like_host(hd[n], "float64", HDIFF_HALO) for n in ("inp", "coeff", "out")},
              {n: Field.like_host(va[n], "float64", VADV_HALO)
               for n in ("ustage", "upos", "utens", "utensstage", "wcon", "out", "ccol", "dcol")})
    sets = [(dev_hd, dev_va), second]
    # uploads and downloads on one stream each (spreading them over four and
    # two streams measured slower: 6.49 against 6.67 GPoints/s; the host link
    # carries 211 GB/s H2D and 193 GB/s D2H alone, ~127 GB/s per direction
    # when both are busy)
    s_ins, s_outs = [Stream()], [Stream()]
    s_in, s_out = s_ins[0], s_outs[0]
    ev_ins = [[Event(), Event()] for _ in s_ins]
    ev_outs = [[Event(), Event()] for _ in s_outs]
    ev_comp = [Event(), Event()]
    in_names = [("hd", "inp"), ("hd", "coeff"), ("va", "ustage"), ("va", "upos"), ("va", "utens"),
                ("va", "utensstage"), ("va", "wcon")]
    out_names = [("hd", "out"), ("va", "out")]

    def wait(st, ev):
        _native.call("sb_stream_wait_event", st.as_parameter, ctypes.c_void_p(ev.handle))

    def pipe_step(n):
        b = n % 2
        fields = {"hd": sets[b][0], "va": sets[b][1]}
        if n >= 2:
            for st in s_ins:
                wait(st, ev_comp[b])  # step n-2 has finished reading this set's inputs
        for q, ((grp, name), (_, pb)) in enumerate(zip(in_names, pinned_in)):
            f = fields[grp][name]
            _native.call("sb_memcpy_async", f.base_ptr, pb.ptr, f.span_bytes, _native.H2D,
                         s_ins[q % len(s_ins)].as_parameter)
        for st, ev in zip(s_ins, ev_ins):
            ev[b].record(st)
            wait(stream, ev[b])
        if n >= 2:
            for ev in ev_outs:
                wait(stream, ev[b])  # step n-2's outputs of this set are downloaded
        kernels.hdiff(fields["hd"]["inp"], fields["hd"]["coeff"], fields["hd"]["out"], stream=stream)
        v = fields["va"]
        kernels.vadv(v["ustage"], v["upos"], v["utens"], v["utensstage"], v["wcon"], out=v["out"], ccol=v["ccol"],
                     dcol=v["dcol"], tune=VADV_TUNE, stream=stream)
        ev_comp[b].record(stream)
        for q, ((grp, name), (_, pb)) in enumerate(zip(out_names, pinned_out)):
            st = s_outs[q % len(s_outs)]
            wait(st, ev_comp[b])
            f = fields[grp][name]
            _native.call("sb_memcpy_async", pb.ptr, f.base_ptr, f.span_bytes, _native.D2H, st.as_parameter)
        for st, ev in zip(s_outs, ev_outs):
            ev[b].record(st)

    for n in range(2):
        pipe_step(n)
    # three timed repetitions of e2e_steps steps, the median reported: the host
    # link is shared with the machine's other GPUs, and a single repetition has
    # measured 3.7 against 6.7 GPoints/s when it met their traffic
    e2e_reps = []
    for _ in range(E2E_REPS):
        _native.synchronize()
        dist.barrier()
        p0, p1 = Event(), Event()
        p0.record(s_in)
        for st in s_ins[1:]:
            wait(st, p0)
        for n in range(e2e_steps):
            pipe_step(n)
        for st in s_outs[1:]:
            last = Event()
            last.record(st)
            wait(s_out, last)
        p1.record(s_out)
        p1.synchronize()
        _native.synchronize()
        e2e_reps.append(dist.max(p0.elapsed(p1)))
    e2e_time = statistics.median(e2e_reps)
    del second, sets

    # ---- the fast float64 step (same inputs, separate outputs), timed the same way
    def fast_step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        kernels.hdiff(dev_hd["inp"], dev_hd["coeff"], dev_hd["out_fast"], compute=FAST_HDIFF_COMPUTE,
                      stream=stream)
        if ev is not None:
            ev[1].record(stream)
        kernels.vadv(dev_va["ustage"], dev_va["upos"], dev_va["utens"], dev_va["utensstage"], dev_va["wcon"],
                     out=dev_va["out_fast"], ccol=dev_va["ccol"], dcol=dev_va["dcol"], compute=FAST_VADV_COMPUTE,
                     tune=FAST_VADV_TUNE, stream=stream)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(args.warmup):
        fast_step()
    stream.synchronize()
    fev = [[Event(), Event(), Event()] for _ in range(args.steps)]
    dist.barrier()
    f0, f1 = Event(), Event()
    f0.record(stream)
    for s in range(args.steps):
        fast_step(fev[s])
    f1.record(stream)
    f1.synchronize()
    fast_elapsed = dist.max(f0.elapsed(f1))
    fast = {"elapsed": fast_elapsed, "t_hdiff": [e[0].elapsed(e[1]) for e in fev],
            "t_vadv": [e[1].elapsed(e[2]) for e in fev]}
    # accuracy against the exact step's outputs (bit-identical to the reference's numpy)
    for name, exact, approx, halo in (("hdiff", "out", "out_fast", HDIFF_HALO),
                                      ("vadv", "out", "out_fast", VADV_HALO)):
        src = dev_hd if name == "hdiff" else dev_va
        host = hd if name == "hdiff" else va
        a = np.empty_like(host[exact])
        b = np.empty_like(host[approx])
        src[exact].download(a)
        src[approx].download(b)
        sl = tuple(slice(h, h + n) for h, n in zip(halo, (NI, NJ, NK)))
        a, b = a[sl], b[sl]
        scale = float(np.max(np.abs(a)))
        big = np.abs(a) >= 1e-2 * np.sqrt(np.mean(a * a))
        pointwise = np.abs(a - b)[big] / np.abs(a)[big]
        fast["err_" + name] = {"max_abs_over_scale": float(np.max(np.abs(a - b))) / scale,
                               "rms_rel": float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(a * a))),
                               "p99_pointwise_rel": float(np.percentile(pointwise, 99)),
                               "p999_pointwise_rel": float(np.percentile(pointwise, 99.9))}

    # ---- STREAM triad calibration (outside the timed region)
    triad = None
    if not args.no_triad:
        bufs = [DeviceBuffer(TRIAD_N * 8) for _ in range(3)]
        a, b, c = (x.ptr for x in bufs)
        kernels.stream_op(_native.STREAM_INIT, "float64", a, b, c, TRIAD_N)
        times = []
        for _ in range(6):
            times.append(kernels.stream_op(_native.STREAM_TRIAD, "float64", a, b, c, TRIAD_N, 3.0, timed=True))
        best = min(times[1:])
        triad = {"n": TRIAD_N, "dtype": "f64", "best_s": best, "gbs": 3 * 8 * TRIAD_N / best / 1e9}
        del bufs

    # ---- fp64 instruction rate (outside the timed region): the exact kernels' ceiling
    fp64_peak = max(kernels.arith_rate(0), kernels.arith_rate(1))

    return {
        "info": info, "elapsed": elapsed_max, "t_hdiff": t_hdiff, "t_vadv": t_vadv, "clocks": clk,
        "gpu_launches": gpu_launches, "e2e_time": e2e_time, "e2e_serial_time": e2e_serial_time,
        "e2e_reps": e2e_reps,
        "e2e_steps": e2e_steps, "h2d": h2d, "d2h": d2h,
        "triad": triad, "fast": fast, "fp64_peak": fp64_peak,
    }


def run_batched(seed=3, n_domains=64, storage="float32", reps=5):
    """64 uneven fp32 domains (half hdiff, half vadv): per-domain launches vs one
    autotuned persistent batched launch replayed from a CUDA graph."""
    from stencil_benchmarks_gb300 import autotune, kernels
    from stencil_benchmarks_gb300.batching import Batch
    from stencil_benchmarks_gb300.device import Event, Stream
    from stencil_benchmarks_gb300.workloads import device_domain, uneven_specs

    specs = uneven_specs(seed=seed, n=n_domains)
    built = [device_domain(s, storage) for s in specs]
    doms = [b[0] for b in built]
    itemsize = 4 if storage == "float32" else (8 if storage == "float64" else 2)
    points = sum(s.points for s in specs)
    cbytes = sum(s.compulsory_bytes(itemsize) for s in specs)
    max_nk = max(s.nk for s in specs)
    stream = Stream()

    def plain(timed=False):
        total = 0.0
        for s, d in zip(specs, doms):
            if s.op == "hdiff":
                t = kernels.hdiff(d.inp, d.coeff, d.out, stream=stream, timed=timed)
            else:
                t = kernels.vadv(d.stage, d.pos, d.tens, d.tensstage, d.wcon, out=d.out, stream=stream, timed=timed)
            total += t or 0.0
        return total

    plain()
    stream.synchronize()
    e0, e1 = Event(), Event()
    t_async = []
    for _ in range(reps):
        e0.record(stream)
        plain()
        e1.record(stream)
        e1.synchronize()
        t_async.append(e0.elapsed(e1))
    t_sync = [plain(timed=True) for _ in range(reps)]
    best, table = autotune.autotune_batch(storage, doms, max_nk)
    batch = Batch(storage, max_domains=n_domains, max_nk=max_nk, **best)
    batch.set(doms)
    t_batch = autotune.time_batch(batch, reps=reps, warmup=2, stream=stream)
    info = batch.info()
    stream.synchronize()
    checked = verify_batched(specs, built, storage)
    ta, ts = statistics.median(t_async), statistics.median(t_sync)
    return {
        "workload": f"{n_domains} uneven domains (half hdiff, half vadv), ni,nj in {{32..512 step 32}}, "
                    f"nk in [40,137], {storage}, seed {seed}",
        "points": points, "compulsory_bytes": cbytes,
        "plain_back_to_back": {"ms": ta * 1e3, "gpoints_s": points / ta / 1e9, "hbm_gbs": cbytes / ta / 1e9},
        "plain_each_synchronised": {"ms": ts * 1e3, "gpoints_s": points / ts / 1e9, "hbm_gbs": cbytes / ts / 1e9},
        "batched_graph": {"ms": t_batch * 1e3, "gpoints_s": points / t_batch / 1e9, "hbm_gbs": cbytes / t_batch / 1e9,
                          "items": info["items"], "grid": info["grid"], "block": info["block"],
                          "workspace_bytes": info["workspace_bytes"]},
        "speedup_vs_back_to_back": ta / t_batch,
        "speedup_vs_each_synchronised": ts / t_batch,
        "autotuned": best, "candidates_timed": len(table),
        "verified": all(ok for _, ok in checked),
        "verified_domains": [f"{what}: {ok}" for what, ok in checked],
    }


def verify_batched(specs, built, storage):
    """Compare the batch's outputs of the tallest and the widest domain bit for
    bit with a per-domain launch of the plain kernel into a fresh field."""
    from stencil_benchmarks_gb300 import _native, kernels
    from stencil_benchmarks_gb300.device import Field

    def interior(host, spec, halo):
        return np.ascontiguousarray(host[halo[0]:halo[0] + spec.ni, halo[1]:halo[1] + spec.nj,
                                         halo[2]:halo[2] + spec.nk])

    def download(field, like):
        span = int(np.sum((np.array(like.shape) - 1) * np.array(like.strides))) + like.itemsize
        out = np.ndarray(like.shape, dtype=like.dtype, strides=like.strides, buffer=np.zeros(span, dtype=np.uint8))
        field.download(out)
        return out

    tall = max(range(len(specs)), key=lambda q: (specs[q].nk, specs[q].points))
    wide = max(range(len(specs)), key=lambda q: (specs[q].ni * specs[q].nj, specs[q].nk))
    results = []
    for what, q in (("tallest", tall), ("widest", wide)):
        spec, (dom, dev, host) = specs[q], built[q]
        halo = dev["out"].halo
        got = interior(download(dev["out"], host["out"]), spec, halo)
        fresh = Field.like_host(host["out"], storage, halo)
        if spec.op == "hdiff":
            kernels.hdiff(dom.inp, dom.coeff, fresh)
        else:
            kernels.vadv(dom.stage, dom.pos, dom.tens, dom.tensstage, dom.wcon, out=fresh)
        _native.synchronize()
        want = interior(download(fresh, host["out"]), spec, halo)
        same = got.tobytes() == want.tobytes()
        results.append((f"{what} {spec.op} {spec.ni}x{spec.nj}x{spec.nk}", bool(same)))
    return results


SERVE_RATES = (1000.0, 5000.0, 10000.0, 20000.0, 50000.0)


def run_served(n_requests=10000, rates=SERVE_RATES, seed=11, float64_compute="float64", mode="batched"):
    """The serving workload: n_requests requests (hdiff / vadv 50/50, ni, nj
    log-uniform in [32, 1024] rounded to 32, nk in [40, 137], fp64 / fp32 /
    bf16-storage at 20/60/20 %, 150 GB budget) at each Poisson arrival rate;
    "batched" packs queued requests into graph replays of the persistent
    kernels, "plain" launches one kernel per request (same admission, slots
    and streams)."""
    from stencil_benchmarks_gb300 import serving

    server = serving.Server(budget_bytes=150e9, max_batch=64, slots_per_form=3, float64_compute=float64_compute,
                            mode=mode)
    # warm-up: enough requests that every slot of every form has launched (and
    # captured its graph) before the measured rates
    serving.run_load(server, serving.request_specs(1024, seed=seed + 1000), rate=1e6)
    out = []
    for rate in rates:
        util = GpuUtilSampler()
        util.start()
        stats = serving.run_load(server, serving.request_specs(n_requests, seed=seed), rate=rate)
        stats["gpu_util_pct"] = util.stop()
        out.append(stats)
    server.close()
    return out


def served_precision_errors(n=12, seed=97):
    """Max |err| / max |exact| and the pointwise p99 relative error of served
    requests of each precision against the exact float64 computation of the
    same stored inputs (the library's float64 kernels, bit-identical to the
    reference's numpy), on a sample of n requests per precision."""
    from stencil_benchmarks_gb300 import kernels, serving
    from stencil_benchmarks_gb300 import array as sbarray
    from stencil_benchmarks_gb300.device import Field

    reqs = [r for r in serving.request_specs(8 * n, seed=seed, sizes=(32, 512))]
    picked = []
    for form in serving.FORMS:
        picked += [r for r in reqs if r.storage == form][:n]
    server = serving.Server(budget_bytes=40e9, max_batch=16, slots_per_form=2, keep_outputs=True, keep_inputs=True)
    for r in picked:
        server.submit(r)
    server.drain()
    errors = {}
    for form in serving.FORMS:
        worst, p99s = 0.0, []
        for r in (q for q in picked if q.storage == form):
            host = {}
            for name, f in r.fields.items():
                a = np.empty(f.shape, dtype=sbarray.storage_numpy_dtype(form), order="F")
                f.download(a)
                host[name] = (a.astype(np.uint32) << 16).view(np.float32) if form == "bfloat16" else a
            wide = {name: np.asfortranarray(a, dtype=np.float64) for name, a in host.items()}
            dev = {name: Field.like_host(a, "float64", r.fields["out"].halo) for name, a in wide.items()}
            for name, a in wide.items():
                dev[name].upload(a)
            if r.op == "hdiff":
                kernels.hdiff(dev["inp"], dev["coeff"], dev["out"])
            else:
                kernels.vadv(dev["stage"], dev["pos"], dev["tens"], dev["tensstage"], dev["wcon"], out=dev["out"])
            exact = np.empty_like(wide["out"])
            dev["out"].download(exact)
            hi, hj, hk = r.fields["out"].halo
            sl = (slice(hi, hi + r.ni), slice(hj, hj + r.nj), slice(hk, hk + r.nk))
            got, want = np.asarray(wide["out"][sl], np.float64), exact[sl]
            scale = float(np.max(np.abs(want))) or 1.0
            worst = max(worst, float(np.max(np.abs(got - want))) / scale)
            big = np.abs(want) >= 1e-2 * np.sqrt(np.mean(want * want))
            p99s.append(float(np.percentile(np.abs(got - want)[big] / np.abs(want)[big], 99)))
            server.release(r)
        errors[form] = {"requests": n, "max_abs_over_scale": worst, "p99_pointwise_rel": max(p99s) if p99s else 0.0}
    server.close()
    return errors


def cpu_baseline_sample(threads=None):
    """Time the C restatement on the full 512x512x80 hdiff+vadv fp64 step."""
    from oracle import cport

    hd, va = make_inputs(seed=7)
    if threads:
        cport.set_threads(threads)
    n_threads = cport.max_threads()
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        cport.hdiff(hd["inp"], hd["coeff"], hd["out"], (NI, NJ, NK), HDIFF_HALO)
        cport.vadv(va["ustage"], va["upos"], va["utens"], va["utensstage"], va["wcon"], (NI, NJ, NK), VADV_HALO,
                   out=va["out"])
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return {
        "value": 2 * POINTS / t / 1e9, "unit": UNIT, "cores": n_threads, "kind": "port",
        "sample": f"full 512x512x80 hdiff+vadv fp64 step, median of {len(times)} runs "
                  f"(oracle/csrc/oracle.c, OpenMP, {n_threads} threads, {os.cpu_count()} host cores)",
        "seconds_per_step": t,
    }


# The reference's own CPU backends (stencils/openmp/horizontal_diffusion.py:50-138,
# stencils/openmp/vertical_advection.py:53-82, stencils/numpy/horizontal_diffusion.py:39-56),
# run through its own Benchmark classes: each renders its C++ template and
# compiles it with g++ -fopenmp -Ofast -march=native at setup.
REF_HDIFF = ("Rolling", "OnTheFlyVec", "OnTheFly")
REF_VADV = ("KInnermostVec", "KInnermost")


def reference_instances(hd, va):
    """Construct the reference's OpenMP hdiff and vadv benchmarks on the bench's
    seeded inputs: {"hdiff": {name: instance}, "vadv": {...}}; raises if the
    reference cannot be loaded or its code does not compile here."""
    from stencil_benchmarks_gb300 import host

    host.load()
    from stencil_benchmarks.benchmarks_collection.stencils.openmp import horizontal_diffusion as ref_hd
    from stencil_benchmarks.benchmarks_collection.stencils.openmp import vertical_advection as ref_va

    out = {"hdiff": {}, "vadv": {}}
    # the reference writes each generated source into ./benchmarks_source_code
    # before compiling it: construct in a scratch directory, not the checkout
    with tempfile.TemporaryDirectory() as scratch, contextlib.chdir(scratch):
        _construct_reference(ref_hd, ref_va, hd, va, out)
    return out


def _construct_reference(ref_hd, ref_va, hd, va, out):
    for name in REF_HDIFF:
        b = getattr(ref_hd, name)(domain=(NI, NJ, NK), halo=HDIFF_HALO, dtype="float64", verify=False)
        for f in ("inp", "coeff"):
            getattr(b._data[0], f)[...] = hd[f]
        out["hdiff"][name] = b
    for name in REF_VADV:
        b = getattr(ref_va, name)(domain=(NI, NJ, NK), halo=VADV_HALO, dtype="float64", verify=False)
        for f in ("ustage", "upos", "utens", "utensstage", "wcon"):
            getattr(b._data[0], f)[...] = va[f]
        out["vadv"][name] = b


def reference_backends(runs=3):
    """Median kernel time (the reference's own timer) of each reference CPU
    backend on the bench's step, and the numpy single-thread hdiff."""
    hd, va = make_inputs(seed=7)
    result = {"threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())), "cpu": _cpu_model()}
    try:
        inst = reference_instances(hd, va)
    except Exception as err:  # noqa: BLE001 - reported, the port still runs
        result["unavailable"] = f"{type(err).__name__}: {err}"[:300]
        return result
    for kind, group in inst.items():
        for name, b in group.items():
            b.run()
            result[f"openmp_{kind}_{name}_ms"] = 1e3 * statistics.median(b.run()["time"] for _ in range(runs))
    for kind in ("hdiff", "vadv"):
        best = min(inst[kind], key=lambda n: result[f"openmp_{kind}_{n}_ms"])
        result[f"best_{kind}"] = best
    step = result[f"openmp_hdiff_{result['best_hdiff']}_ms"] + result[f"openmp_vadv_{result['best_vadv']}_ms"]
    result["openmp_step_ms"] = step
    result["openmp_value"] = 2 * POINTS / (step * 1e-3) / 1e9
    from stencil_benchmarks.benchmarks_collection.stencils.numpy import horizontal_diffusion as np_hd

    b = np_hd.OnTheFly(domain=(NI, NJ, NK), halo=HDIFF_HALO, dtype="float64", verify=False)
    b._data[0].inp[...] = hd["inp"]
    b._data[0].coeff[...] = hd["coeff"]
    result["numpy_hdiff_OnTheFly_ms"] = 1e3 * b.run()["time"]
    return result


def _cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def run_reference(args, dist):
    """--impl reference: the reference's own OpenMP backends (best hdiff + best
    vadv) on the host cores, each step timed by the reference's own timer;
    the C port if the reference cannot be loaded or compiled here."""
    if dist.rank != 0:
        return 0
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    hd, va = make_inputs(seed=7)
    try:
        inst = reference_instances(hd, va)
    except Exception as err:  # noqa: BLE001
        print(f"reference backends unavailable ({type(err).__name__}: {err}); timing the C port", file=sys.stderr)
        return run_reference_port(args, hd, va, dist)
    best = {}
    for kind, group in inst.items():
        timings = {}
        for name, b in group.items():
            for _ in range(max(1, args.warmup)):
                b.run()
            timings[name] = statistics.median(b.run()["time"] for _ in range(3))
        best[kind] = min(timings, key=timings.get)
    h, v = inst["hdiff"][best["hdiff"]], inst["vadv"][best["vadv"]]
    step_times = []
    for _ in range(args.steps):
        step_times.append(h.run()["time"] + v.run()["time"])
    elapsed = sum(step_times)
    value = 2 * POINTS * args.steps / elapsed / 1e9
    threads = int(os.environ["OMP_NUM_THREADS"])
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64, workload distributions)",
        "config": dict(CONFIG),
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": threads, "kind": "reference",
            "sample": f"every step is the full 512x512x80 fp64 step: the reference's OpenMP "
                      f"horizontal_diffusion.{best['hdiff']} + vertical_advection.{best['vadv']} (fastest of "
                      f"{'/'.join(REF_HDIFF)} and {'/'.join(REF_VADV)}), run through the reference's own Benchmark "
                      f"classes and timers, {threads} threads on {os.cpu_count()} host cores ({_cpu_model()})",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference_port(args, hd, va, dist):
    """The C restatement of the reference arithmetic on the host cores."""
    from oracle import cport

    n_threads = cport.max_threads()
    for _ in range(args.warmup):
        cport.hdiff(hd["inp"], hd["coeff"], hd["out"], (NI, NJ, NK), HDIFF_HALO)
        cport.vadv(va["ustage"], va["upos"], va["utens"], va["utensstage"], va["wcon"], (NI, NJ, NK), VADV_HALO,
                   out=va["out"])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cport.hdiff(hd["inp"], hd["coeff"], hd["out"], (NI, NJ, NK), HDIFF_HALO)
        cport.vadv(va["ustage"], va["upos"], va["utens"], va["utensstage"], va["wcon"], (NI, NJ, NK), VADV_HALO,
                   out=va["out"])
    elapsed = time.perf_counter() - t0
    value = 2 * POINTS * args.steps / elapsed / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64, workload distributions)",
        "config": dict(CONFIG),
        "cpu_baseline": {
            "value": value, "unit": UNIT, "cores": n_threads, "kind": "port",
            "sample": "every step is the full 512x512x80 hdiff+vadv fp64 step on the host cores "
                      "(C restatement of the reference arithmetic, OpenMP)",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the timed CPU baseline")
    ap.add_argument("--no-triad", action="store_true", help="skip the STREAM triad calibration")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-domains comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the serving-loop measurement")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        res = run_gpu(args, dist)
        if dist.rank != 0:
            return 0
        peak, peak_kind = measured_peaks()
        t_h = statistics.mean(res["t_hdiff"])
        t_v = statistics.mean(res["t_vadv"])
        dominant = "vadv" if t_v >= t_h else "hdiff"
        t_dom = max(t_h, t_v)
        achieved = compulsory_bytes(dominant) / t_dom / 1e9
        traffic = ncu_traffic().get(dominant)
        value = 2 * POINTS * args.steps * dist.world / res["elapsed"] / 1e9
        e2e_value = 2 * POINTS * res["e2e_steps"] * dist.world / res["e2e_time"] / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["elapsed"] / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded PCG64, workload distributions)",
            "config": dict(CONFIG),
            "device": {"name": res["info"]["name"], "sm_count": res["info"]["sm_count"]},
            "gpu_launches": res["gpu_launches"],
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": res["h2d"],
                    "d2h_bytes_per_step": res["d2h"], "steps": res["e2e_steps"],
                    "path": "C ABI: pinned host -> sb_memcpy_async -> sb_hdiff + sb_vadv -> pinned host; "
                            "uploads, kernels and downloads on three streams over two device sets; "
                            "host link measured alone: 211 GB/s H2D, 193 GB/s D2H",
                    "timing": f"median of {len(res['e2e_reps'])} timed repetitions of {res['e2e_steps']} steps",
                    "rep_values": [2 * POINTS * res["e2e_steps"] * dist.world / t / 1e9 for t in res["e2e_reps"]],
                    "serial_value": 2 * POINTS * res["e2e_steps"] * dist.world / res["e2e_serial_time"] / 1e9},
            "roofline": {"bound": "hbm", "limiter": "fp64 pipe: exact fp64 arithmetic runs at 1/73 of the fp32 "
                                                   "rate on GB300 (0.52 Tops/s measured)",
                         "kernel": dominant, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic, "algorithmic_bytes": compulsory_bytes(dominant),
                         "fp64_pipe": {
                             "what": "algorithmic fp64 operations per second (hdiff 16, vadv 27 per point, a divide "
                                     "counted once) / the fp64 add-or-FMA instruction rate measured in this run; can "
                                     "exceed 1 where exact power-of-two scales and the limiter's sign tests run on "
                                     "the integer pipe",
                             "achieved": FP64_OPS[dominant] * POINTS / t_dom, "peak": res["fp64_peak"],
                             "unit": "op/s", "frac": FP64_OPS[dominant] * POINTS / t_dom / res["fp64_peak"],
                             "hdiff_frac": FP64_OPS["hdiff"] * POINTS / t_h / res["fp64_peak"],
                             "vadv_frac": FP64_OPS["vadv"] * POINTS / t_v / res["fp64_peak"]}},
            "kernels": {
                "hdiff": {"ms": t_h * 1e3, "gpoints_s": POINTS / t_h / 1e9,
                          "hbm_gbs": compulsory_bytes("hdiff") / t_h / 1e9,
                          "frac_of_" + peak_kind: compulsory_bytes("hdiff") / t_h / 1e9 / peak},
                "vadv": {"ms": t_v * 1e3, "gpoints_s": POINTS / t_v / 1e9,
                         "hbm_gbs": compulsory_bytes("vadv") / t_v / 1e9,
                         "frac_of_" + peak_kind: compulsory_bytes("vadv") / t_v / 1e9 / peak},
            },
            "stream_triad": res["triad"],
            "clocks": res["clocks"],
        }
        fast = res["fast"]
        fh, fv = statistics.mean(fast["t_hdiff"]), statistics.mean(fast["t_vadv"])
        line["fast_f64"] = {
            "what": "same step and inputs; hdiff fixed-point sums + one fp64 FMA (fp64 rounding level), vadv "
                    "float-pair arithmetic (~48-bit significand); not bit-identical to the reference, and the "
                    "float-pair vadv is not held to 1e-10 of the field scale in near-singular columns (errors "
                    "against the exact step: max |err| / max |exact| and pointwise relative p99 / p99.9 over "
                    "|exact| >= 1e-2 rms)",
            "value": 2 * POINTS * args.steps * dist.world / fast["elapsed"] / 1e9, "unit": UNIT,
            "ms_per_step": fast["elapsed"] / args.steps * 1e3,
            "hdiff": {"compute": FAST_HDIFF_COMPUTE, "ms": fh * 1e3, "gpoints_s": POINTS / fh / 1e9,
                      "hbm_gbs": compulsory_bytes("hdiff") / fh / 1e9,
                      "frac_of_" + peak_kind: compulsory_bytes("hdiff") / fh / 1e9 / peak,
                      "traffic": ncu_traffic().get("hdiff_fixed64"), "error_vs_exact": fast["err_hdiff"]},
            "vadv": {"compute": FAST_VADV_COMPUTE, "tune": FAST_VADV_TUNE, "ms": fv * 1e3,
                     "gpoints_s": POINTS / fv / 1e9, "hbm_gbs": compulsory_bytes("vadv") / fv / 1e9,
                     "frac_of_" + peak_kind: compulsory_bytes("vadv") / fv / 1e9 / peak,
                     "traffic": ncu_traffic().get("vadv_f32x2"), "error_vs_exact": fast["err_vadv"]},
            "gpu_launches": 2 * args.steps,
        }
        if res["triad"]:
            line["stream_triad"]["frac_of_" + peak_kind] = res["triad"]["gbs"] / peak
        # serving first: its latencies are measured in a process that has not
        # yet created and torn down the autotuner's many batch objects
        if not args.no_served:
            batched = run_served()
            plain = run_served(mode="plain")
            sat_b = max(r["throughput_req_s"] for r in batched)
            sat_p = max(r["throughput_req_s"] for r in plain)
            line["served"] = {
                "workload": "10,000 requests per rate, Poisson arrivals; hdiff/vadv 50/50, ni,nj log-uniform in "
                            "[32,1024] rounded to 32, nk in [40,137], fp64/fp32/bf16-storage 20/60/20 %, 150 GB "
                            "budget, fields generated on the device",
                "batched": batched, "plain": plain,
                "saturation_req_s": {"batched": sat_b, "plain": sat_p, "ratio": sat_b / sat_p},
                "p99_ms_at_5k": {"batched": batched[1]["p99_ms"], "plain": plain[1]["p99_ms"]},
                "error_vs_exact_fp64": served_precision_errors(),
            }
            line["served_fast_f64"] = {
                "what": "float64 requests with fixed-point hdiff and float-pair vadv (within 1e-12 / 1e-10 of "
                        "the field scale); float32 and bfloat16 requests unchanged",
                "rates": run_served(rates=(5000.0, 20000.0), float64_compute="fixed64")}
        if not args.no_batched:
            line["batched"] = run_batched()
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample()
            line["cpu_baseline"]["reference_backends"] = reference_backends()
        print(json.dumps(line), flush=True)
        return 0
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
