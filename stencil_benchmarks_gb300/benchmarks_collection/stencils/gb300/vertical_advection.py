"""Vertical advection on GB300: ``sbench stencils gb300 vertical-advection <impl>``.

Counterpart of stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/
vertical_advection.py:39-73.  Every class derives from the reference's
``VerticalAdvectionStencil`` (fields, verification, ``data_size``).  The
fields and the in-place update of
``utensstage`` (and, with ``all_components``, ``vtensstage``/``wtensstage``)
are the reference's; each component is one ``sb_vadv`` launch, with wcon read
at the column shifted by (1, 0), (0, 1) and (0, 0) for u, v and w
(stencils/base.py:475-483), except in ``TensorMem``, where ``sb_vadv3`` solves
the three in one launch (the reference's fused kernel:
cuda_hip/templates/vertical_advection_localmemmerged.j2).

* ``SharedMem``     -- factors in shared memory, inputs staged with cp.async;
* ``GlobalScratch`` -- factors in the ``ccol``/``dcol`` fields at each
  column's own position;
* ``Slab``          -- persistent threads with their factors in compact,
  L2-resident slabs of ``ccol``/``dcol`` (fastest float64 and float-pair
  form);
* ``NoAlloc``       -- factors in the library's static scratch array
  (``sb_vadv_noalloc``), for callers that cannot allocate device memory;
* ``TensorMem``     -- float32 compute: rows staged per warp, factors in the
  SM's tensor memory (one persistent block per SM; fastest float32 and, with
  16-byte-multiple level strides, bfloat16 form).
"""

from __future__ import annotations

import ctypes
import warnings

import numpy as np

from stencil_benchmarks.benchmark import Parameter, ParameterError
from stencil_benchmarks.benchmarks_collection.stencils import base

from .... import _native, kernels
from ....device import _stream_arg
from .mixin import StencilMixin

_SHIFTS = {"u": (1, 0), "v": (0, 1), "w": (0, 0)}


class VerticalAdvectionMixin(StencilMixin):
    block_size = Parameter("threads per block along i and j", (32, 1))
    unroll_factor = Parameter("levels of inputs kept in flight (1, 2, 4 or 8)", 4, choices=[1, 2, 4, 8])

    def check_parameters(self):
        super().check_parameters()
        if self.compute_dtype == "fixed64":
            raise ParameterError("fixed64 compute is provided for horizontal diffusion only")
        if self.domain[2] < 2 and int(np.prod(self.domain)) > 0:
            raise ParameterError("vertical advection needs at least 2 levels")
        if self.verify and self.dry_runs:
            warnings.warn(
                "using --dry-runs together with verification might lead to false negatives for "
                "stencils with read-write fields"
            )

    @property
    def compulsory_bytes(self):
        ni, nj, nk = self.domain
        comps = 3 if self.all_components else 1
        # per component: stage, pos, tens, tensstage read + tensstage written; wcon once (+ shifted column/row)
        return (comps * 5 * ni * nj * nk + (ni + 1) * (nj + 1) * nk) * self.dtype_size

    def components(self, fields):
        named = dict(zip(self.args, fields))
        comps = ["u", "v", "w"] if self.all_components else ["u"]
        for c in comps:
            yield c, [named[f"{c}{n}"] for n in ("stage", "pos", "tens", "tensstage")], named

    def launch_component(self, f, named, shift, timed):
        raise NotImplementedError

    def launch(self, fields, timed):
        total = 0.0
        for c, f, named in self.components(fields):
            t = self.launch_component(f, named, _SHIFTS[c], timed)
            total += t or 0.0
        return total if timed else None


class SharedMem(VerticalAdvectionMixin, base.VerticalAdvectionStencil):
    def tune(self):
        return _native.tune(variant=_native.VADV_SMEM, block_x=self.block_size[0], block_y=self.block_size[1],
                            unroll=self.unroll_factor)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.VADV_SMEM, block_x=bx, block_y=by, unroll=u)
                                for bx, by in ((32, 1), (64, 1), (32, 2)) for u in (2, 4, 8)]

    def launch_component(self, f, named, shift, timed):
        return kernels.vadv(*f, named["wcon"], shift, compute=self.compute, tune=self.current_tune(), timed=timed)


class GlobalScratch(VerticalAdvectionMixin, base.VerticalAdvectionStencil):
    block_size = Parameter("threads per block along i and j", (64, 1))
    unroll_factor = Parameter("levels of inputs kept in flight (1, 2, 4 or 8)", 2, choices=[1, 2, 4, 8])

    def check_parameters(self):
        super().check_parameters()
        if self.dtype_size != {"float64": 8, "float32": 4, "float32x2": 8}[self.compute]:
            raise ParameterError("GlobalScratch keeps the factors in ccol/dcol: storage and compute types must match")

    def tune(self):
        return _native.tune(variant=_native.VADV_GLOBAL, block_x=self.block_size[0], block_y=self.block_size[1],
                            unroll=self.unroll_factor)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.VADV_GLOBAL, block_x=bx, block_y=1, unroll=u)
                                for bx in (32, 64, 128) for u in (1, 2, 4)]

    def launch_component(self, f, named, shift, timed):
        return kernels.vadv(*f, named["wcon"], shift, ccol=named["ccol"], dcol=named["dcol"], compute=self.compute,
                            tune=self.current_tune(), timed=timed)


class Slab(VerticalAdvectionMixin, base.VerticalAdvectionStencil):
    block_size = Parameter("threads per block along i (32 or 64), persistent blocks per SM (0: the library's "
                           "choice: 24 when the float64 products run in integer arithmetic, otherwise as many as "
                           "keep the factor slabs within half of L2)", (32, 0))
    unroll_factor = Parameter("levels of inputs kept in flight (1 with 32-thread blocks, 2, 4 or 8)", 1,
                              choices=[1, 2, 4, 8])

    def check_parameters(self):
        super().check_parameters()
        if self.unroll_factor == 1 and self.block_size[0] != 32:
            raise ParameterError("Slab keeps one level in flight with 32-thread blocks only")
        if self.dtype_size != {"float64": 8, "float32": 4, "float32x2": 8}.get(self.compute, 0) and not (
                self.dtype == "bfloat16" and self.compute == "float32"):
            raise ParameterError("Slab stages its ccol/dcol factors in ring entries: compute type as wide as storage")
        if self.block_size[0] not in (32, 64):
            raise ParameterError("Slab blocks have 32 or 64 threads")

    def tune(self):
        return _native.tune(variant=_native.VADV_SLAB, block_x=self.block_size[0], k_per_cta=self.block_size[1],
                            unroll=self.unroll_factor)

    def tune_candidates(self):
        return [self.tune()] + [_native.tune(variant=_native.VADV_SLAB, block_x=bx, k_per_cta=per, unroll=u)
                                for bx in (32, 64) for per in (0, 8, 16)
                                for u in ((1, 2, 4, 8) if bx == 32 else (2, 4, 8))]

    def launch_component(self, f, named, shift, timed):
        return kernels.vadv(*f, named["wcon"], shift, ccol=named["ccol"], dcol=named["dcol"], compute=self.compute,
                            tune=self.current_tune(), timed=timed)


class NoAlloc(VerticalAdvectionMixin, base.VerticalAdvectionStencil):
    def launch_component(self, f, named, shift, timed):
        stage, pos, tens, tensstage = f
        ni, nj, nk = self.domain
        t = ctypes.c_double(0.0)
        _native.call(
            "sb_vadv_noalloc", _native.storage_code(self.dtype), _native.storage_code(self.compute),
            *(ctypes.c_void_p(x.interior_ptr) for x in (stage, pos, tens, tensstage, named["wcon"], tensstage)),
            ni, nj, nk, *stage.strides, shift[0], shift[1], _stream_arg(None), ctypes.byref(t) if timed else None,
        )
        return t.value if timed else None


class TensorMem(VerticalAdvectionMixin, base.VerticalAdvectionStencil):
    dtype = Parameter("data type: float32 or bfloat16 (float32 compute)", "float32")
    unroll_factor = Parameter("levels of inputs kept in flight (4, 8 or 16)", 8, choices=[4, 8, 16])

    def check_parameters(self):
        super().check_parameters()
        if self.compute != "float32":
            raise ParameterError("TensorMem keeps float32 factors in tensor memory: float32 compute only")
        if self.domain[2] > 256:
            raise ParameterError("TensorMem holds at most 256 levels per column")

    def tune(self):
        return _native.tune(variant=_native.VADV_TMEM, unroll=self.unroll_factor)

    def tune_candidates(self):
        return [_native.tune(variant=_native.VADV_TMEM, unroll=u) for u in (4, 8, 16)]

    def launch_component(self, f, named, shift, timed):
        return kernels.vadv(*f, named["wcon"], shift, compute=self.compute, tune=self.current_tune(), timed=timed)

    def launch(self, fields, timed):
        if not self.all_components:
            return super().launch(fields, timed)
        # u, v and w in one launch (sb_vadv3): each column group's three
        # solves in turn, wcon from HBM once
        comps = [f for _, f, _ in self.components(fields)]
        named = dict(zip(self.args, fields))
        return kernels.vadv3(comps, named["wcon"], compute=self.compute, tune=self.current_tune(), timed=timed)
