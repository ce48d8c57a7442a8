"""The GB300 backend: common part of every stencil benchmark.

Counterpart of the reference's cuda_hip ``StencilMixin``
(stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/mixin.py:50-175).
The concrete classes derive from this mixin and from the reference's own
``Stencil`` subclasses (stencil_benchmarks/benchmarks_collection/stencils/
base.py), so the reference allocates and fills the host fields, runs and
verifies them (``Stencil.run``, ``verify_stencil``) and reports
``bandwidth``; this mixin only implements ``run_stencil``: copy the host
fields to the device, launch the prebuilt sm_103a kernel, time the launch
with CUDA events ("gpu") or the host clock ("wall"), copy the fields back and
return ``{"time": seconds}`` plus ``gpoints_per_s`` and ``hbm_gbs``
(compulsory bytes over the time).  The device fields are allocated once in
``setup`` with the host fields' layout, instead of on every run.

Additions to the reference's parameters: ``compute_dtype`` (the storage type
stays ``dtype``), ``device`` and ``autotune``.  ``dtype`` also accepts
"bfloat16" (host fields hold the 16-bit patterns as uint16, filled from the
reference's U[0, 1) distribution rounded to nearest even); the reference's
numpy verification has no bfloat16 type, so bfloat16 storage needs
``verify=False``.  A compute type wider than the storage (float32 fields,
float64 arithmetic) is more accurate than the reference's check, which
recomputes in the storage type: in ill-conditioned vertical-advection columns
the two can differ by more than the reference's float32 tolerance.
"""

from __future__ import annotations

import statistics
import time

import numpy as np
from stencil_benchmarks.benchmark import Benchmark, ExecutionError, Parameter, ParameterError
from stencil_benchmarks.tools import array as ref_array

from .... import _native
from ....device import Field

BFLOAT16 = "bfloat16"


def _round_to_bf16_bits(values: np.ndarray) -> np.ndarray:
    bits = values.astype(np.float32).view(np.uint32).astype(np.uint64)
    return ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)


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

    # -- bfloat16 storage on top of the reference's field allocation ----------

    @property
    def dtype_size(self):
        return 2 if self.dtype == BFLOAT16 else np.dtype(self.dtype).itemsize

    def alloc_field(self, domain_with_halo, layout, index_to_align):
        if self.dtype != BFLOAT16:
            return super().alloc_field(domain_with_halo, layout, index_to_align)
        # the reference's layout/alignment rule on a 2-byte element type
        return ref_array.alloc_array(domain_with_halo, np.uint16, layout, self.alignment,
                                     index_to_align=index_to_align, apply_offset=self.offset_allocations)

    def random_field(self):
        if self.dtype != BFLOAT16:
            return super().random_field()
        data = self.empty_field()
        data[...] = _round_to_bf16_bits(np.random.default_rng().random(data.shape))
        return data

    # -- tuning -------------------------------------------------------------

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

    # -- setup / run ----------------------------------------------------------

    def check_parameters(self):
        """Reject unsupported parameter values before any field is allocated."""
        if self.dtype not in ("float64", "float32", BFLOAT16):
            raise ParameterError(f"unsupported dtype {self.dtype!r}: float64, float32 or bfloat16")
        if self.dtype == BFLOAT16 and self.verify:
            raise ParameterError("bfloat16 storage: the reference's numpy verification has no bfloat16 type, "
                                 "run with verify=False")
        if self.compute_dtype == "float32" and self.dtype == "float64":
            raise ParameterError("float64 storage with float32 compute is not provided")
        if self.compute_dtype in ("float32x2", "fixed64") and self.dtype != "float64":
            raise ParameterError(f"{self.compute_dtype} compute needs float64 storage")

    def setup(self):
        self.check_parameters()
        if self.dry_runs < 0:
            raise ParameterError("dry_runs must be non-negative")
        try:
            ndev = _native.device_count()
        except _native.NativeLibraryError as err:
            raise ParameterError(str(err)) from err
        if self.device >= ndev:
            raise ParameterError(f"CUDA device {self.device} not available ({ndev} device(s))")
        super().setup()
        _native.call("sb_set_device", self.device)
        self._device_fields = [Field.like_host(host, self.dtype, self.halo) for host in self._data[0]]
        self._picked_tune = None
        if self.autotune:
            self._picked_tune = (self._pick_tune(),)

    @property
    def compute(self) -> str:
        if self.compute_dtype == "auto":
            return "float64" if self.dtype == "float64" else "float32"
        return self.compute_dtype

    @property
    def compulsory_bytes(self) -> int:
        """Bytes a perfect kernel moves: each input read once, each output written once."""
        raise NotImplementedError

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
        result = {
            "time": elapsed,
            "gpoints_per_s": float(np.prod(self.domain)) / elapsed / 1e9,
            "hbm_gbs": self.compulsory_bytes / elapsed / 1e9,
        }
        if self.autotune:
            result["tune"] = self.describe_tune(self.current_tune())
        return result
