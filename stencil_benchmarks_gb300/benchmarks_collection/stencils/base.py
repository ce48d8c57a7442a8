"""Stencil base classes: the reference's ``Stencil`` contract without its CPU math.

Same Parameters, field allocation, data-set cycling and ``run()`` result as
stencil_benchmarks/benchmarks_collection/stencils/base.py:45-166; the
concrete stencil classes declare the same ``args`` and ``data_size`` as the
reference (base.py:168-347).  Differences, all deliberate:

* fields are filled from a seeded generator (``seed`` parameter) instead of
  the reference's unseeded ``random_fill`` -- same U[0, 1) distribution;
* ``dtype`` also accepts "bfloat16" (host arrays hold bit patterns);
* ``verify_stencil`` delegates to the verifier registered for the stencil's
  kind (``stencil_benchmarks_gb300.verification``), because this package has
  no CPU implementation; with ``verify=True`` and no verifier registered,
  construction fails with ParameterError;
* ``run()`` adds ``gpoints_per_s`` and ``hbm_gbs`` (compulsory bytes) to the
  reference's ``time`` and ``bandwidth`` keys.
"""

from __future__ import annotations

import abc
import collections
import copy

import numpy as np

from ... import array as sbarray
from ... import verification
from ...benchmark import Benchmark, ExecutionError, Parameter, ParameterError

STORAGE_TYPES = ("float64", "float32", "bfloat16")


class Stencil(Benchmark):
    domain = Parameter("domain size", (128, 128, 80))
    data_sets = Parameter(
        "number of data sets, if bigger than one, data sets are cycled before "
        "each execution to start with cold cache",
        1,
    )
    halo = Parameter("halo size", (3, 3, 3))
    dtype = Parameter("data type in NumPy format, e.g. float32 or float64 (or bfloat16)", "float64")
    layout = Parameter("data layout, 2 means innermost dimension, 0 outermost", (2, 1, 0))
    alignment = Parameter("data alignment in bytes", 0)
    huge_pages = Parameter("use huge pages", "none", choices=["none", "transparent", "explicit"])
    offset_allocations = Parameter("offset allocated data by some bytes to minimize cache conflicts", False)
    verify = Parameter("enable verification", True)
    seed = Parameter("seed of the random field initialisation", 0)

    #: verification kind looked up in ``verification`` (set by subclasses)
    stencil_kind: str = ""

    def setup(self):
        super().setup()
        if any(h < 0 for h in self.halo):
            raise ParameterError(f"negative halo size given ({self.halo})")
        if tuple(sorted(self.layout)) != (0, 1, 2):
            raise ParameterError(f"invalid layout specification {self.layout}")
        if self.dtype not in STORAGE_TYPES:
            raise ParameterError(f"unsupported dtype {self.dtype!r}; choose one of {STORAGE_TYPES}")
        if self.alignment < 0:
            raise ParameterError(f"negative alignment given ({self.alignment} bytes)")
        if self.alignment % self.dtype_size != 0:
            raise ParameterError(
                f"alignment ({self.alignment} bytes) not divisible by dtype size ({self.dtype_size} bytes)"
            )
        if self.huge_pages != "none":
            raise ParameterError("huge-page host buffers are not provided by this backend")
        if any(d < 0 for d in self.domain):
            raise ParameterError(f"negative domain size given ({self.domain})")
        if self.data_sets < 1:
            raise ParameterError("data_sets must be at least 1")
        if self.verify and verification.get(self.stencil_kind) is None:
            raise ParameterError(
                f"verify=True needs a CPU verifier for '{self.stencil_kind}': run with verify=False, or "
                "register one (stencil_benchmarks_gb300.reference_bridge.install() uses the reference's own "
                "numpy verification when stencil_benchmarks is installed)"
            )
        self._rng = np.random.Generator(np.random.PCG64(self.seed))
        fields = collections.namedtuple("StencilData", self.args)
        self._data = [fields._make(self.random_field() for _ in self.args) for _ in range(self.data_sets)]
        self._run = 0

    # -- fields ---------------------------------------------------------------

    def alloc_field(self, domain_with_halo, layout, index_to_align):
        return sbarray.alloc_array(
            domain_with_halo, self.dtype, layout, self.alignment, index_to_align=index_to_align,
            apply_offset=self.offset_allocations,
        )

    def empty_field(self):
        return self.alloc_field(self.domain_with_halo, self.layout, self.halo)

    def random_field(self):
        data = self.empty_field()
        values = self._rng.random(data.shape)
        if self.dtype == "bfloat16":
            bits = values.astype(np.float32).view(np.uint32).astype(np.uint64)
            data[...] = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
        else:
            data[...] = values
        return data

    @property
    def dtype_size(self):
        return sbarray.element_size(self.dtype)

    @property
    def domain_with_halo(self):
        return tuple(d + 2 * h for d, h in zip(self.domain, self.halo))

    @property
    def strides(self):
        return tuple(s // self.dtype_size for s in self._data[0][0].strides)

    @property
    def data_size(self):
        return len(self.args) * int(np.prod(self.domain)) * self.dtype_size

    @property
    def compulsory_bytes(self):
        """Bytes a perfect kernel moves (each input read once, output written once)."""
        return self.data_size

    def inner_slice(self, shift=None, expand=None):
        shift = [0] * len(self.domain) if shift is None else shift
        if expand is None:
            expand = [0] * len(self.domain)
        elif isinstance(expand, int):
            expand = [expand] * len(self.domain)
        return tuple(
            slice(h + s - e, h + d + s + e) for d, h, s, e in zip(self.domain, self.halo, shift, expand)
        )

    # -- contract -------------------------------------------------------------

    @abc.abstractmethod
    def run_stencil(self, data):
        """Run on ``data`` (namedtuple of host fields, updated in place); return {"time": s}."""

    def verify_stencil(self, data_before, data_after):
        verifier = verification.get(self.stencil_kind)
        if verifier is None:
            raise ExecutionError(f"no verifier registered for '{self.stencil_kind}'")
        verifier(self, data_before, data_after)

    @property
    @abc.abstractmethod
    def args(self):
        """Names of the fields, in the order ``run_stencil`` receives them."""

    def run(self):
        index = self._run % self.data_sets
        if self.verify:
            data_before = copy.deepcopy(self._data[index])
        result = self.run_stencil(self._data[index])
        if self.verify:
            self.verify_stencil(data_before, self._data[index])
        self._run += 1
        assert "time" in result and result["time"] > 0
        assert "bandwidth" not in result
        result["bandwidth"] = self.data_size / result["time"] / 1e9
        result["gpoints_per_s"] = float(np.prod(self.domain)) / result["time"] / 1e9
        result["hbm_gbs"] = self.compulsory_bytes / result["time"] / 1e9
        return result


class BasicStencil(Stencil):
    @property
    def args(self):
        return "inp", "out"

    @property
    def compulsory_bytes(self):
        return 2 * int(np.prod(self.domain)) * self.dtype_size


class EmptyStencil(BasicStencil):
    """The reference's launch-overhead probe: no memory traffic, nothing to verify."""

    stencil_kind = "empty"

    @property
    def compulsory_bytes(self):
        return 0


class CopyStencil(BasicStencil):
    stencil_kind = "copy"


class OnesidedAverageStencil(BasicStencil):
    stencil_kind = "onesided_average"
    axis = Parameter("axis along which to average", 0, choices=[0, 1, 2])

    def setup(self):
        super().setup()
        if self.halo[self.axis] < 1:
            raise ParameterError(f"positive halo size required along axis {self.axis} (given halo: {self.halo})")


class SymmetricAverageStencil(OnesidedAverageStencil):
    stencil_kind = "symmetric_average"


class LaplacianStencil(BasicStencil):
    stencil_kind = "laplacian"
    along_x = Parameter("include x-axis in Laplacian", True)
    along_y = Parameter("include y-axis in Laplacian", True)
    along_z = Parameter("include z-axis in Laplacian", False)

    def setup(self):
        super().setup()
        axes = (self.along_x, self.along_y, self.along_z)
        if any(h < 1 for h, a in zip(self.halo, axes) if a):
            raise ParameterError(f"positive horizontal halo size required (given halo: {self.halo})")


class HorizontalDiffusionStencil(Stencil):
    stencil_kind = "horizontal_diffusion"

    def setup(self):
        super().setup()
        if any(h < 2 for h in self.halo[:2]):
            raise ParameterError(f"horizontal halo size must be at least 2 (given halo: {self.halo})")

    @property
    def args(self):
        return "inp", "coeff", "out"

    @property
    def data_size(self):
        # the reference's accounting (base.py:270-274), k-halo of 4 included
        return (2 * int(np.prod(self.domain)) + int(np.prod(np.array(self.domain) + 4))) * self.dtype_size

    @property
    def compulsory_bytes(self):
        ni, nj, nk = self.domain
        return ((ni + 4) * (nj + 4) * nk + 2 * ni * nj * nk) * self.dtype_size


class VerticalAdvectionStencil(Stencil):
    stencil_kind = "vertical_advection"
    all_components = Parameter(
        "advect all velocity components (like in the COSMO dycore) "
        "instead of the u component (like in the GridTools benchmark)",
        False,
    )

    def setup(self):
        super().setup()
        if self.halo[0] < 1 or (self.all_components and any(h < 1 for h in self.halo)):
            raise ParameterError(f"positive halo size required (given halo: {self.halo})")
        if self.domain[2] < 2 and int(np.prod(self.domain)) > 0:
            raise ParameterError("vertical advection needs at least 2 levels")

    @property
    def args(self):
        u = ("ustage", "upos", "utens", "utensstage")
        v = ("vstage", "vpos", "vtens", "vtensstage")
        w = ("wstage", "wpos", "wtens", "wtensstage")
        common = ("wcon", "ccol", "dcol", "datacol")
        return u + common if not self.all_components else u + v + w + common

    @property
    def data_size(self):
        # the reference's accounting (base.py:339-347): ccol/dcol traffic included
        reads, writes = (7, 3) if not self.all_components else (15, 5)
        return (reads + writes) * int(np.prod(self.domain)) * self.dtype_size

    @property
    def compulsory_bytes(self):
        ni, nj, nk = self.domain
        comps = 3 if self.all_components else 1
        # per component: stage, pos, tens, tensstage read + tensstage written; wcon once (+ shifted column/row)
        return (comps * 5 * ni * nj * nk + (ni + 1) * (nj + 1) * nk) * self.dtype_size
