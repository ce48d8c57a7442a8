"""Host reproduction of the device field generator and oracle checks of
served requests (test infrastructure)."""

from __future__ import annotations

import numpy as np

from oracle import stencils as ora
from stencil_benchmarks_gb300 import serving

_G = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def fill_values(seed, count, lo, hi, storage):
    """What sb_fill_batch writes: storage values (bf16 as uint16 bits)."""
    with np.errstate(over="ignore"):
        e = np.arange(count, dtype=np.uint64)
        z = np.uint64(seed) + (e + np.uint64(1)) * _G
        u = (splitmix64(z) >> np.uint64(11)).astype(np.float64) * 2.0**-53
    v = lo + (hi - lo) * u
    if storage == "float64":
        return v
    if storage == "float32":
        return v.astype(np.float32)
    return ora.f32_to_bf16_bits(v.astype(np.float32))


def request_inputs(req):
    """Halo'd input arrays of a request, as the device generated them (F-order)."""
    shape, _, halo = serving.field_layout(req.op, req.ni, req.nj, req.nk)
    specs = serving.HDIFF_FIELDS if req.op == "hdiff" else serving.VADV_FIELDS
    out = {}
    count = int(np.prod(shape))
    for q, (name, lo, hi) in enumerate(specs):
        if lo is None:
            continue
        vals = fill_values(serving.field_seed(req.seed, q), count, lo, hi, req.storage)
        out[name] = vals.reshape(shape, order="F")
    return out, halo


def expected_output(req):
    """Oracle result of a request on its interior, in storage type."""
    fields, halo = request_inputs(req)
    compute = np.float64 if req.storage == "float64" else np.float32
    if req.storage == "bfloat16":
        fields = {n: ora.bf16_bits_to_f32(a.ravel(order="F")).reshape(a.shape, order="F")
                  for n, a in fields.items()}
    fields = {n: np.asarray(a, dtype=compute) for n, a in fields.items()}
    domain = (req.ni, req.nj, req.nk)
    if req.op == "hdiff":
        res = ora.hdiff(fields["inp"], fields["coeff"], domain, halo)
    else:
        res = ora._vadv_component(fields["stage"], fields["pos"], fields["tens"], fields["tensstage"],
                                  fields["wcon"], domain, halo, 1, 0)
    if req.storage == "bfloat16":
        return ora.f32_to_bf16_bits(np.asarray(res, dtype=np.float32)).reshape(res.shape)
    return np.asarray(res).astype(req.storage)


def download_output(req):
    """The request's output interior from the device."""
    from stencil_benchmarks_gb300.array import storage_numpy_dtype

    f = req.fields["out"]
    host = np.empty(f.shape, dtype=storage_numpy_dtype(req.storage), order="F")
    f.download(host)
    hi, hj, hk = f.halo
    return host[hi:hi + req.ni, hj:hj + req.nj, hk:hk + req.nk]
