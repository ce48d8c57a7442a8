"""Basic stencils on GB300: ``sbench stencils gb300 basic <impl>``.

Counterpart of stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/basic.py:101-132
(empty, copy, one-sided / symmetric average, Laplacian), running ``sb_empty``,
``sb_copy``, ``sb_average`` and ``sb_laplacian``.
"""

from __future__ import annotations

from .... import _native, kernels
from ....benchmark import Parameter
from .. import base
from .mixin import StencilMixin


class BasicStencilMixin(StencilMixin):
    block_size = Parameter("threads per block along i and j", (128, 2))

    def tune(self):
        return _native.tune(block_x=self.block_size[0], block_y=self.block_size[1])


class Empty(BasicStencilMixin, base.EmptyStencil):
    def launch(self, fields, timed):
        return kernels.empty(fields[0], tune=self.tune(), timed=timed)


class Copy(BasicStencilMixin, base.CopyStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.copy(inp, out, tune=self.tune(), timed=timed)


class OnesidedAverage(BasicStencilMixin, base.OnesidedAverageStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.average(inp, out, self.axis, False, compute=self.compute, tune=self.tune(), timed=timed)


class SymmetricAverage(BasicStencilMixin, base.SymmetricAverageStencil):
    def launch(self, fields, timed):
        inp, out = fields
        return kernels.average(inp, out, self.axis, True, compute=self.compute, tune=self.tune(), timed=timed)


class Laplacian(BasicStencilMixin, base.LaplacianStencil):
    def launch(self, fields, timed):
        inp, out = fields
        along = (self.along_x, self.along_y, self.along_z)
        return kernels.laplacian(inp, out, along, compute=self.compute, tune=self.tune(), timed=timed)
