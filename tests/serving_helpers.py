"""Host reproduction of the device field generator and oracle checks of
served requests (test infrastructure)."""

from __future__ import annotations

import numpy as np

from oracle import stencils as ora
from stencil_benchmarks_gb300 import serving

def lowbias32(x):
    """C. Wellons' lowbias32 hash on uint32 arrays."""
    x = x ^ (x >> np.uint32(16))
    x = x * np.uint32(0x7FEB352D)
    x = x ^ (x >> np.uint32(15))
    x = x * np.uint32(0x846CA68B)
    return x ^ (x >> np.uint32(16))


def _keys(seed):
    with np.errstate(over="ignore"):
        k0 = lowbias32(np.uint32(seed & 0xFFFFFFFF) ^ np.uint32(0xA511E9B3)) | np.uint32(1)
        k1 = lowbias32(np.uint32(seed >> 32) + np.uint32(0x632BE5AB))
        k2 = lowbias32(k0 ^ k1)
    return k0, k1, k2


def _hash(n, k0, k1):
    """H(x(n)) for an array of uint64 indices n."""
    with np.errstate(over="ignore"):
        lo32 = (n & np.uint64(0xFFFFFFFF)).astype(np.uint32)
        hi32 = (n >> np.uint64(32)).astype(np.uint32)
        return lowbias32(lo32 * k0 + k1 + hi32 * np.uint32(0x9E3779B9))


def fill_values(seed, count, lo, hi, storage):
    """What sb_fill_batch writes: storage values (bf16 as uint16 bits)."""
    k0, k1, k2 = _keys(seed)
    lo_f = np.float32(lo)
    span_f = np.float32(np.float64(hi) - np.float64(lo))
    with np.errstate(over="ignore"):
        if storage == "float64":
            h1 = _hash(np.arange(count, dtype=np.uint64), k0, k1)
            h2 = lowbias32(h1 ^ k2)
            k = (h1.astype(np.uint64) << np.uint64(21)) | (h2 >> np.uint32(11)).astype(np.uint64)
            span = np.float64(hi) - np.float64(lo)
            return np.float64(lo) + span * (k.astype(np.float64) * 2.0**-53)
        if storage == "float32":
            h = _hash(np.arange(count, dtype=np.uint64), k0, k1)
            v = lo_f + span_f * ((h >> np.uint32(8)).astype(np.float32) * np.float32(2.0**-24))
            assert v.dtype == np.float32
            return v
        e = np.arange(count, dtype=np.uint64)
        h = _hash(e >> np.uint64(1), k0, k1)
        bits = np.where((e & np.uint64(1)) == 1, h >> np.uint32(16), h & np.uint32(0xFFFF))
        v = lo_f + span_f * (bits.astype(np.float32) * np.float32(2.0**-16))
        assert v.dtype == np.float32
        return ora.f32_to_bf16_bits(v)


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


def expected_output_c(req):
    """``expected_output`` computed by the C oracle (OpenMP; same bits as the
    numpy oracle, which its golden tests pin), for large requests."""
    from oracle import cport

    fields, halo = request_inputs(req)
    compute = np.float64 if req.storage == "float64" else np.float32
    if req.storage == "bfloat16":
        fields = {n: ora.bf16_bits_to_f32(a.ravel(order="F")).reshape(a.shape, order="F")
                  for n, a in fields.items()}
    fields = {n: np.asfortranarray(a, dtype=compute) for n, a in fields.items()}
    domain = (req.ni, req.nj, req.nk)
    first = next(iter(fields.values()))
    out = np.zeros(first.shape, dtype=compute, order="F")
    if req.op == "hdiff":
        cport.hdiff(fields["inp"], fields["coeff"], out, domain, halo)
    else:
        cport.vadv(fields["stage"], fields["pos"], fields["tens"], fields["tensstage"], fields["wcon"], domain, halo,
                   (1, 0), out=out)
    res = out[tuple(slice(h, h + n) for h, n in zip(halo, domain))]
    if req.storage == "bfloat16":
        return ora.f32_to_bf16_bits(np.ascontiguousarray(res, dtype=np.float32)).reshape(res.shape)
    return np.asarray(res).astype(req.storage)
