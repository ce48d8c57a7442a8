"""The GB300 backend: common part of every stencil benchmark.

Counterpart of the reference's cuda_hip ``StencilMixin``
(stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/mixin.py:50-175):
the same ``dry_runs`` / ``timers`` / ``gpu_architecture`` knobs and the same
``run_stencil`` contract -- copy the host fields to the device, launch,
time the launch with CUDA events ("gpu") or the host clock ("wall"), copy the
fields back, return ``{"time": seconds}``.  Instead of rendering and
compiling a kernel per parameter set it calls the prebuilt sm_103a library;
the device fields are allocated once in ``setup`` (same layout as the host
fields) rather than on every run.
"""

from __future__ import annotations

import statistics
import time

from .... import _native
from ....benchmark import Benchmark, ExecutionError, Parameter, ParameterError
from ....device import Field


class StencilMixin(Benchmark):
    gpu_architecture = Parameter("GPU architecture (the library is built for sm_103a)", "sm_103a",
                                 choices=["sm_103a"])
    dry_runs = Parameter("kernel dry-runs before the measurement", 0)
    timers = Parameter("timer type", "gpu", choices=["gpu", "wall"])
    compute_dtype = Parameter(
        "compute type: auto (float64 for float64 storage, else float32), float32, float64, float32x2 "
        "(float-pair arithmetic, float64 storage) or fixed64 (hdiff: fixed-point sums, float64 storage)", "auto",
        choices=["auto", "float32", "float64", "float32x2", "fixed64"],
    )
    device = Parameter("CUDA device index", 0)
    autotune = Parameter("time this implementation's candidate launch shapes on the benchmark's own fields "
                         "during setup and run the fastest (reported as `tune`)", False)

    def tune(self):
        """This implementation's launch shape (None: the library's choice)."""
        return None

    def tune_candidates(self):
        """Launch shapes the autotuner times: this implementation's own family."""
        return [self.tune()]

    def current_tune(self):
        picked = getattr(self, "_picked_tune", None)
        return picked[0] if picked is not None else self.tune()

    def _pick_tune(self):
        fields = self._device_fields
        best, best_t = None, None
        for cand in self.tune_candidates():
            for host, dev in zip(self._data[0], fields):
                dev.upload(host)
            self._picked_tune = (cand,)
            try:
                self.launch(fields, timed=False)
                t = statistics.median(self.launch(fields, timed=True) for _ in range(3))
            except _native.SbError:
                continue
            if best_t is None or t < best_t:
                best, best_t = cand, t
        self._picked_tune = None
        if best_t is None:
            raise ParameterError("autotune: no candidate launch shape runs on this layout")
        return best

    @staticmethod
    def describe_tune(t) -> str:
        if t is None:
            return "library default"
        return " ".join(f"{name}={getattr(t, name)}" for name, _ in t._fields_ if getattr(t, name))

    def setup(self):
        super().setup()
        if self.dry_runs < 0:
            raise ParameterError("dry_runs must be non-negative")
        try:
            ndev = _native.device_count()
        except _native.NativeLibraryError as err:
            raise ParameterError(str(err)) from err
        if self.device >= ndev:
            raise ParameterError(f"CUDA device {self.device} not available ({ndev} device(s))")
        _native.call("sb_set_device", self.device)
        if self.compute_dtype == "float32" and self.dtype == "float64":
            raise ParameterError("float64 storage with float32 compute is not provided")
        if self.compute_dtype in ("float32x2", "fixed64") and self.dtype != "float64":
            raise ParameterError(f"{self.compute_dtype} compute needs float64 storage")
        if self.compute_dtype == "fixed64" and self.stencil_kind != "horizontal_diffusion":
            raise ParameterError("fixed64 compute is provided for horizontal diffusion only")
        self._device_fields = [Field.like_host(host, self.dtype, self.halo) for host in self._data[0]]
        self._picked_tune = None
        if self.autotune:
            self._picked_tune = (self._pick_tune(),)

    @property
    def compute(self) -> str:
        if self.compute_dtype == "auto":
            return "float64" if self.dtype == "float64" else "float32"
        return self.compute_dtype

    def launch(self, fields, timed: bool):
        """Launch the stencil on device ``fields``; with ``timed`` return seconds."""
        raise NotImplementedError

    def run_stencil(self, data):
        _native.call("sb_set_device", self.device)
        fields = self._device_fields
        for host, dev in zip(data, fields):
            dev.upload(host)
        try:
            for _ in range(self.dry_runs):
                self.launch(fields, timed=False)
            if self.timers == "gpu":
                elapsed = self.launch(fields, timed=True)
            else:
                _native.synchronize()
                start = time.perf_counter()
                self.launch(fields, timed=False)
                _native.synchronize()
                elapsed = time.perf_counter() - start
        except _native.SbError as err:
            raise ExecutionError(str(err)) from err
        for host, dev in zip(data, fields):
            dev.download(host)
        if self.autotune:
            return {"time": elapsed, "tune": self.describe_tune(self.current_tune())}
        return {"time": elapsed}
