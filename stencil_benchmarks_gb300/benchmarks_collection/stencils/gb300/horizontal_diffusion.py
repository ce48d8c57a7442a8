"""Horizontal diffusion on GB300: ``sbench stencils gb300 horizontal-diffusion <impl>``.

Counterpart of stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/
horizontal_diffusion.py:40-128 (whose implementations are named after their
algorithm).  Both classes run ``sb_hdiff``:

* ``JScan`` -- warp j-march with shuffles (the default, HBM-efficient form);
* ``Tile``  -- shared-memory k-plane tiles (fewest fp64 operations).
"""

from __future__ import annotations

from .... import _native, kernels
from ....benchmark import Parameter, ParameterError
from .. import base
from .mixin import StencilMixin


class HorizontalDiffusionMixin(StencilMixin):
    def tune(self):
        raise NotImplementedError

    def launch(self, fields, timed):
        inp, coeff, out = fields
        return kernels.hdiff(inp, coeff, out, compute=self.compute, tune=self.tune(), timed=timed)


class JScan(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    block_size = Parameter("warps per block (28 columns each) and rows per block", (4, 32))
    unroll_factor = Parameter("rows loaded per batch (1, 2, 4 or 8)", 4, choices=[1, 2, 4, 8])
    k_per_block = Parameter("k-planes per block", 1)

    def setup(self):
        super().setup()
        if not 1 <= self.block_size[0] <= 8 or self.block_size[1] < 1:
            raise ParameterError("block_size: 1..8 warps and at least 1 row")

    def tune(self):
        return _native.tune(variant=_native.HDIFF_JSCAN, block_y=self.block_size[0], tile_y=self.block_size[1],
                            k_per_cta=self.k_per_block, unroll=self.unroll_factor)


class Tile(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    block_size = Parameter("threads along i, threads along j, rows per tile", (64, 4, 16))
    k_per_block = Parameter("k-planes per block", 4)

    def setup(self):
        super().setup()
        bx, by, ty = self.block_size
        if (bx, by) not in {(32, 4), (32, 8), (64, 2), (64, 4), (64, 8), (128, 2), (128, 4)}:
            raise ParameterError("block_size[:2] must be one of 32x4, 32x8, 64x2, 64x4, 64x8, 128x2, 128x4")
        if ty < by:
            raise ParameterError("rows per tile must be at least the threads along j")

    def tune(self):
        bx, by, ty = self.block_size
        return _native.tune(variant=_native.HDIFF_TILE, block_x=bx, block_y=by, tile_y=ty,
                            k_per_cta=self.k_per_block)
