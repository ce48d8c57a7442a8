"""Use the reference's own numpy verification when stencil_benchmarks is installed.

The reference's ``Stencil`` subclasses verify with plain methods that only
read ``self.domain``, ``self.halo``, ``self.inner_slice()`` and the stencil's
parameters (stencil_benchmarks/benchmarks_collection/stencils/base.py:180-501);
this package's stencils have the same attributes, so those methods can run
unchanged on them.  ``install()`` registers them with
``stencil_benchmarks_gb300.verification`` and returns True, or returns False
when the reference cannot be imported.  bfloat16 fields are not supported by
the reference's verification (numpy has no bfloat16).
"""

from __future__ import annotations

from . import verification

_KINDS = {
    "copy": "CopyStencil",
    "onesided_average": "OnesidedAverageStencil",
    "symmetric_average": "SymmetricAverageStencil",
    "laplacian": "LaplacianStencil",
    "horizontal_diffusion": "HorizontalDiffusionStencil",
    "vertical_advection": "VerticalAdvectionStencil",
}


def install() -> bool:
    try:
        from stencil_benchmarks.benchmarks_collection.stencils import base as ref_base
        from stencil_benchmarks.tools import validation as ref_validation
    except Exception:  # noqa: BLE001 - any import problem means "reference not available"
        return False

    from .validation import ValidationError

    def make(cls_name):
        method = getattr(ref_base, cls_name).verify_stencil

        def verifier(stencil, before, after):
            if stencil.dtype == "bfloat16":
                raise ValidationError("the reference's verification has no bfloat16 support")
            try:
                method(stencil, before, after)
            except ref_validation.ValidationError as err:
                raise ValidationError(*err.args) from err

        return verifier

    for kind, cls_name in _KINDS.items():
        verification.register(kind, make(cls_name))
    return True
