"""STREAM on GB300: ``sbench stream gb300 native``.

Counterpart of stencil_benchmarks/benchmarks_collection/stream/cuda_hip.py:41-144
and its kernels/driver (stream/cuda_hip.j2:132-345): arrays a = 1, b = 2,
c = 0 are initialised on the device, then ``ntimes`` rounds of copy (c = a),
scale (b = s*c), add (c = a + b) and triad (a = b + s*c) with s = 3 are each
timed with CUDA events.  The first round is dropped; the result is one dict
per kernel with the reference's keys ``name``, ``bandwidth`` (MB/s of the best
round, 2 or 3 arrays moved), ``avg-time``, ``time`` (the best) and
``max-time``.  With ``verify`` the final arrays are checked against the
scalar recurrence with the reference's criterion (average relative error at
most 1e-6 for float32, 1e-13 for float64); a failure raises the reference's
``ValidationError``.  The class derives from the reference's ``Benchmark``,
so it registers as ``stream gb300 native``.
"""

from __future__ import annotations

import numpy as np
from stencil_benchmarks.benchmark import Benchmark, ExecutionError, Parameter, ParameterError
from stencil_benchmarks.tools.validation import ValidationError

from ... import _native, kernels
from ...device import DeviceBuffer, copy_to_host


class Native(Benchmark):
    array_size = Parameter("number of elements in arrays", 10000000)
    ntimes = Parameter("number of runs", 10)
    block_size = Parameter("threads per block (0: the grid shape's default)", 0)
    grid = Parameter("grid shape: a few blocks per SM striding over the arrays, one block per chunk of "
                     "block_size x unroll_factor vectors, or the library's choice", "auto",
                     choices=["auto", "stride", "chunk"])
    dtype = Parameter("data type in NumPy format, e.g. float32 or float64", "float64",
                      choices=["float32", "float64"])
    unroll_factor = Parameter("16-byte vectors per thread per iteration (0: the grid shape's default)", 0,
                              choices=[0, 1, 2, 4, 8])
    streaming_stores = Parameter("use streaming (evict-first) store instructions", False)
    verify = Parameter("verify results", True)
    device = Parameter("CUDA device index", 0)

    def setup(self):
        super().setup()
        if self.ntimes < 2:
            raise ParameterError("ntimes must be at least 2 (the first round is dropped)")
        limit = 1024 if self.grid == "chunk" else 512
        if self.array_size < 1 or self.block_size % 32 or not 0 <= self.block_size <= limit:
            raise ParameterError(f"array_size >= 1 and block_size 0 or a multiple of 32 up to {limit} required")
        try:
            ndev = _native.device_count()
        except _native.NativeLibraryError as err:
            raise ParameterError(str(err)) from err
        if self.device >= ndev:
            raise ParameterError(f"CUDA device {self.device} not available ({ndev} device(s))")
        _native.call("sb_set_device", self.device)
        itemsize = np.dtype(self.dtype).itemsize
        self._bufs = [DeviceBuffer(self.array_size * itemsize) for _ in range(3)]
        grid = {"auto": 0, "stride": _native.STREAM_GRID_STRIDE, "chunk": _native.STREAM_GRID_CHUNK}[self.grid]
        self._tune = _native.tune(variant=grid, block_x=self.block_size, unroll=self.unroll_factor,
                                  flags=1 if self.streaming_stores else 0)

    def run(self):
        _native.call("sb_set_device", self.device)
        a, b, c = (x.ptr for x in self._bufs)
        n, dt = self.array_size, self.dtype
        names = ("copy", "scale", "add", "triad")
        ops = (_native.STREAM_COPY, _native.STREAM_SCALE, _native.STREAM_ADD, _native.STREAM_TRIAD)
        times = {name: [] for name in names}
        try:
            kernels.stream_op(_native.STREAM_INIT, dt, a, b, c, n)
            for _ in range(self.ntimes):
                for name, op in zip(names, ops):
                    times[name].append(kernels.stream_op(op, dt, a, b, c, n, 3.0, tune=self._tune, timed=True))
        except _native.SbError as err:
            raise ExecutionError(str(err)) from err
        itemsize = np.dtype(dt).itemsize
        results = []
        for name in names:
            t = times[name][1:]
            arrays = 2 if name in ("copy", "scale") else 3
            results.append({
                "name": name,
                "bandwidth": 1e-6 * arrays * itemsize * n / min(t),
                "avg-time": sum(t) / len(t),
                "time": min(t),
                "max-time": max(t),
            })
        if self.verify:
            self._check(a, b, c)
        return results

    def _check(self, a, b, c):
        t = np.dtype(self.dtype).type
        aj, bj, cj, s = t(1), t(2), t(0), t(3)
        for _ in range(self.ntimes):
            cj = aj
            bj = s * cj
            cj = aj + bj
            aj = bj + s * cj
        eps = 1e-6 if self.dtype == "float32" else 1e-13
        for label, ptr, want in (("a", a, aj), ("b", b, bj), ("c", c, cj)):
            if not np.isfinite(want):
                raise ValidationError("expected value is infinite, ntimes too large for verification")
            host = np.empty(self.array_size, dtype=self.dtype)
            copy_to_host(host, ptr)
            err = float(np.mean(np.abs(host.astype(np.float64) - float(want)))) / abs(float(want))
            if err > eps:
                bad = int(np.count_nonzero(np.abs(host / want - 1) > eps))
                raise ValidationError(f"failed validation on array {label}[]: average relative error {err:.3g}, "
                                      f"{bad} elements off by more than {eps:g}")
