"""Horizontal diffusion on GB300: ``sbench stencils gb300 horizontal-diffusion <impl>``.

Counterpart of stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/
horizontal_diffusion.py:40-128 (whose implementations are named after their
algorithm).  Every class derives from the reference's
``HorizontalDiffusionStencil`` (fields, verification, ``data_size``) and runs
``sb_hdiff``:

* ``JScan``      -- warp j-march with shuffles (HBM-efficient float32 form);
* ``Tile``       -- shared-memory k-plane tiles (fewest fp64 operations);
* ``TmaTile``    -- the tiles with each k-plane brought in by the tensor
  memory accelerator, double-buffered (fastest exact float64 form; needs
  j/k strides that are multiples of 16 bytes, hence alignment 64 by default);
* ``VectorScan`` -- the j-march with several columns per lane moved as one
  aligned vector (fastest bfloat16-storage and float-pair form).
"""

from __future__ import annotations

from stencil_benchmarks.benchmark import Parameter, ParameterError
from stencil_benchmarks.benchmarks_collection.stencils import base

from .... import _native, kernels
from .mixin import StencilMixin


class HorizontalDiffusionMixin(StencilMixin):
    def tune(self):
        raise NotImplementedError

    @property
    def compulsory_bytes(self):
        ni, nj, nk = self.domain
        return ((ni + 4) * (nj + 4) * nk + 2 * ni * nj * nk) * self.dtype_size

    def launch(self, fields, timed):
        inp, coeff, out = fields
        return kernels.hdiff(inp, coeff, out, compute=self.compute, tune=self.current_tune(), timed=timed)


class JScan(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    block_size = Parameter("warps per block (28 columns each) and rows per block", (4, 32))
    unroll_factor = Parameter("rows loaded per batch (1, 2, 4 or 8)", 4, choices=[1, 2, 4, 8])
    k_per_block = Parameter("k-planes per block", 1)

    def check_parameters(self):
        super().check_parameters()
        if not 1 <= self.block_size[0] <= 8 or self.block_size[1] < 1:
            raise ParameterError("block_size: 1..8 warps and at least 1 row")

    def tune(self):
        return _native.tune(variant=_native.HDIFF_JSCAN, block_y=self.block_size[0], tile_y=self.block_size[1],
                            k_per_cta=self.k_per_block, unroll=self.unroll_factor)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.HDIFF_JSCAN, block_y=nw, tile_y=ty, k_per_cta=1, unroll=u)
                                for nw in (1, 2, 4) for ty in (16, 32, 64) for u in (2, 4)]


class Tile(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    block_size = Parameter("threads along i, threads along j, rows per tile", (64, 4, 16))
    k_per_block = Parameter("k-planes per block", 4)

    def check_parameters(self):
        super().check_parameters()
        bx, by, ty = self.block_size
        if (bx, by) not in {(32, 4), (32, 8), (64, 2), (64, 4), (64, 8), (128, 2), (128, 4)}:
            raise ParameterError("block_size[:2] must be one of 32x4, 32x8, 64x2, 64x4, 64x8, 128x2, 128x4")
        if ty < by:
            raise ParameterError("rows per tile must be at least the threads along j")

    def tune(self):
        bx, by, ty = self.block_size
        return _native.tune(variant=_native.HDIFF_TILE, block_x=bx, block_y=by, tile_y=ty,
                            k_per_cta=self.k_per_block)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.HDIFF_TILE, block_x=bx, block_y=by, tile_y=ty, k_per_cta=k)
                                for bx, by in ((128, 4), (64, 4), (64, 8), (128, 2)) for ty in (8, 16, 32)
                                for k in (2, 4)]


class TmaTile(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    alignment = Parameter("data alignment in bytes (rows padded so that TMA can describe them)", 64)
    block_size = Parameter("threads along i, threads along j, rows per tile", (128, 4, 16))
    k_per_block = Parameter("k-planes per block (double-buffered)", 1)

    def check_parameters(self):
        super().check_parameters()
        bx, by, ty = self.block_size
        if (bx, by) not in {(32, 8), (64, 4), (64, 8), (128, 2), (128, 4)}:
            raise ParameterError("block_size[:2] must be one of 32x8, 64x4, 64x8, 128x2, 128x4")
        if not by <= ty <= 252:
            raise ParameterError("rows per tile must be in [threads along j, 252]")

    def tune(self):
        bx, by, ty = self.block_size
        return _native.tune(variant=_native.HDIFF_TMA, block_x=bx, block_y=by, tile_y=ty,
                            k_per_cta=self.k_per_block)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.HDIFF_TMA, block_x=bx, block_y=by, tile_y=ty, k_per_cta=k)
                                for bx, by in ((128, 4), (64, 4), (64, 8), (128, 2)) for ty in (8, 12, 16, 32)
                                for k in (2, 4)]


class VectorScan(HorizontalDiffusionMixin, base.HorizontalDiffusionStencil):
    block_size = Parameter("strip width (32 x columns per lane; 0: 16 bytes per lane), warps per block, "
                           "rows per warp", (0, 1, 16))
    unroll_factor = Parameter("rows loaded per batch (1, 2, 4 or 8)", 1, choices=[1, 2, 4, 8])
    k_per_block = Parameter("k-planes per block", 1)

    def check_parameters(self):
        super().check_parameters()
        width, nw, rows = self.block_size
        if width not in (0, 64, 128, 256) or not 1 <= nw <= 8 or rows < 1:
            raise ParameterError("block_size: width 0, 64, 128 or 256, 1..8 warps, at least 1 row")

    def tune(self):
        width, nw, rows = self.block_size
        if width == 0:
            width = {8: 64, 4: 128, 2: 128}[self.dtype_size]
        return _native.tune(variant=_native.HDIFF_VSCAN, block_x=width, block_y=nw, tile_y=rows,
                            k_per_cta=self.k_per_block, unroll=self.unroll_factor)

    def tune_candidates(self):
        widths = {8: (64,), 4: (64, 128), 2: (128, 256)}[self.dtype_size]
        return [self.tune()] + [_native.tune(variant=_native.HDIFF_VSCAN, block_x=w, block_y=nw, tile_y=ty,
                                             k_per_cta=1, unroll=u)
                                for w in widths for nw in (1, 2, 4) for ty in (16, 32) for u in (1, 4)]
