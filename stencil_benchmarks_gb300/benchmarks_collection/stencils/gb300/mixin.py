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
        return {"time": elapsed}
