"""CPU verifiers for the benchmark classes, built on the oracle.

The product package has no CPU implementation; its ``Stencil.run()`` asks
``stencil_benchmarks_gb300.verification`` for a verifier.  The tests install
these, which recompute each stencil with the oracle (in the stencil's compute
type, on the values its storage holds) and compare with the reference's
tolerances (``stencil_benchmarks_gb300.validation``).  Read-only fields must
be unchanged, exactly as the reference checks.
"""

from __future__ import annotations

import numpy as np

from oracle import stencils as ora
from stencil_benchmarks_gb300 import validation, verification


def _compute_view(arr, stencil):
    compute = stencil.compute if hasattr(stencil, "compute") else (
        "float64" if stencil.dtype == "float64" else "float32")
    if stencil.dtype == "bfloat16":
        vals = ora.bf16_bits_to_f32(np.ascontiguousarray(arr)).reshape(arr.shape)
    else:
        vals = np.array(arr)
    return vals.astype(np.float64 if compute in ("float64", "float32x2", "fixed64") else np.float32)


def _to_storage(values, stencil):
    if stencil.dtype == "bfloat16":
        return ora.f32_to_bf16_bits(np.asarray(values, dtype=np.float32)).reshape(np.shape(values))
    return np.asarray(values).astype(stencil.dtype)


def _unchanged(before, after, names):
    for n in names:
        validation.check_equality(n, getattr(after, n), getattr(before, n))


def _check_out(stencil, name, after, expected):
    got = getattr(after, name)[stencil.inner_slice()]
    validation.check_equality(name, np.ascontiguousarray(got), _to_storage(expected, stencil), storage=stencil.dtype)


def _basic(fn):
    def verifier(stencil, before, after):
        _unchanged(before, after, ["inp"])
        inp = _compute_view(before.inp, stencil)
        _check_out(stencil, "out", after, fn(stencil, inp))

    return verifier


def _hdiff(stencil, before, after):
    _unchanged(before, after, ["inp", "coeff"])
    exp = ora.hdiff(_compute_view(before.inp, stencil), _compute_view(before.coeff, stencil), stencil.domain,
                    stencil.halo)
    _check_out(stencil, "out", after, exp)


def _vadv(stencil, before, after):
    readonly = [n for n in stencil.args if n.endswith(("stage", "pos", "tens")) and not n.endswith("tensstage")]
    _unchanged(before, after, readonly + ["wcon"])
    fields = {n: _compute_view(getattr(before, n), stencil) for n in stencil.args}
    exp = ora.vadv(fields, stencil.domain, stencil.halo, stencil.all_components)
    for name, values in exp.items():
        _check_out(stencil, name, after, values)


def install():
    verification.register("copy", _basic(lambda s, inp: ora.copy(inp, s.domain, s.halo)))
    verification.register("onesided_average",
                          _basic(lambda s, inp: ora.onesided_average(inp, s.domain, s.halo, s.axis)))
    verification.register("symmetric_average",
                          _basic(lambda s, inp: ora.symmetric_average(inp, s.domain, s.halo, s.axis)))
    verification.register("laplacian", _basic(
        lambda s, inp: ora.laplacian(inp, s.domain, s.halo, (s.along_x, s.along_y, s.along_z))))
    verification.register("horizontal_diffusion", _hdiff)
    verification.register("vertical_advection", _vadv)
