"""Basic stencils on GB300: ``sbench stencils gb300 basic <impl>``.

Counterpart of stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/basic.py:101-132
(empty, copy, one-sided / symmetric average, Laplacian), running ``sb_empty``,
``sb_copy``, ``sb_average`` and ``sb_laplacian``.  Every class derives from
the reference's stencil class of the same name (fields, verification).
"""

from __future__ import annotations

import numpy as np
from stencil_benchmarks.benchmark import Parameter, ParameterError
from stencil_benchmarks.benchmarks_collection.stencils import base

from .... import _native, kernels
from .mixin import StencilMixin


class BasicStencilMixin(StencilMixin):
    block_size = Parameter("threads per block along i and j", (128, 2))

    def check_parameters(self):
        super().check_parameters()
        if self.compute_dtype == "fixed64":
            raise ParameterError("fixed64 compute is provided for horizontal diffusion only")

    def tune(self):
        return _native.tune(block_x=self.block_size[0], block_y=self.block_size[1])

    @property
    def compulsory_bytes(self):
        return 2 * int(np.prod(self.domain)) * self.dtype_size


class AverageMixin(BasicStencilMixin):
    def check_parameters(self):
        super().check_parameters()
        if self.halo[self.axis] < 1:
            raise ParameterError(f"positive halo size required along axis {self.axis} (given halo: {self.halo})")


class Empty(BasicStencilMixin, base.EmptyStencil):
    @property
    def compulsory_bytes(self):
        return 0

    def launch(self, fields, timed):
        return kernels.empty(fields[0], tune=self.tune(), timed=timed)


class Copy(BasicStencilMixin, base.CopyStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.copy(inp, out, tune=self.tune(), timed=timed)


class OnesidedAverage(AverageMixin, base.OnesidedAverageStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.average(inp, out, self.axis, False, compute=self.compute, tune=self.tune(), timed=timed)


class SymmetricAverage(AverageMixin, base.SymmetricAverageStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.average(inp, out, self.axis, True, compute=self.compute, tune=self.tune(), timed=timed)


class Laplacian(BasicStencilMixin, base.LaplacianStencil):
    def launch(self, fields, timed):
        inp, out = fields
        along = (self.along_x, self.along_y, self.along_z)
        return kernels.laplacian(inp, out, along, compute=self.compute, tune=self.tune(), timed=timed)
