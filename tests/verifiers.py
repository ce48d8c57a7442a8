"""Oracle checks of a benchmark's fields after a run (test infrastructure).

The benchmark classes are verified by the reference's own numpy
``verify_stencil`` (``np.isclose``).  These helpers check the same run
against the oracle more strictly: bit for bit in the stencil's compute type
(the oracle run on the values the storage holds, rounded once to storage),
and for bfloat16 storage, which the reference's verification cannot take.
Read-only fields must be unchanged.
"""

from __future__ import annotations

import numpy as np

from oracle import stencils as ora

_EXACT = {"float64": np.uint64, "float32": np.uint32, "bfloat16": np.uint16}


def compute_view(arr, stencil):
    if stencil.dtype == "bfloat16":
        vals = ora.bf16_bits_to_f32(np.ascontiguousarray(arr)).reshape(arr.shape)
    else:
        vals = np.array(arr)
    wide = stencil.compute in ("float64", "float32x2", "fixed64")
    return vals.astype(np.float64 if wide else np.float32)


def to_storage(values, stencil):
    if stencil.dtype == "bfloat16":
        return ora.f32_to_bf16_bits(np.asarray(values, dtype=np.float32)).reshape(np.shape(values))
    return np.asarray(values).astype(stencil.dtype)


def _same_bits(name, got, want, dtype):
    got = np.ascontiguousarray(got)
    want = np.ascontiguousarray(want)
    bits = _EXACT[dtype]
    same = got.view(bits) == want.view(bits)
    if dtype != "bfloat16":
        same |= np.isnan(got) & np.isnan(want)
    assert same.all(), f"{name}: {np.count_nonzero(~same)} points differ from the oracle"


def expected_outputs(stencil, before):
    kind = type(stencil).__module__.rsplit(".", 1)[-1]
    if kind == "horizontal_diffusion":
        exp = ora.hdiff(compute_view(before.inp, stencil), compute_view(before.coeff, stencil), stencil.domain,
                        stencil.halo)
        return {"out": exp}
    if kind == "vertical_advection":
        fields = {n: compute_view(getattr(before, n), stencil) for n in stencil.args}
        return ora.vadv(fields, stencil.domain, stencil.halo, stencil.all_components)
    inp = compute_view(before.inp, stencil)
    name = type(stencil).__name__
    if name == "Copy":
        return {"out": ora.copy(inp, stencil.domain, stencil.halo)}
    if name == "OnesidedAverage":
        return {"out": ora.onesided_average(inp, stencil.domain, stencil.halo, stencil.axis)}
    if name == "SymmetricAverage":
        return {"out": ora.symmetric_average(inp, stencil.domain, stencil.halo, stencil.axis)}
    if name == "Laplacian":
        along = (stencil.along_x, stencil.along_y, stencil.along_z)
        return {"out": ora.laplacian(inp, stencil.domain, stencil.halo, along)}
    assert name == "Empty", name
    return {}


def check_bit_exact(stencil, before, after):
    """Outputs bit-identical to the oracle in the compute type; inputs unchanged."""
    outputs = expected_outputs(stencil, before)
    for name in stencil.args:
        if name in outputs or name in ("ccol", "dcol", "datacol"):
            continue
        _same_bits(name, getattr(after, name), getattr(before, name), stencil.dtype)
    sl = stencil.inner_slice()
    for name, values in outputs.items():
        _same_bits(name, getattr(after, name)[sl], to_storage(values, stencil), stencil.dtype)
