"""Helpers shared by the GPU tests: seeded fields in the reference's layout,
upload/download through the C ABI, and oracle evaluation per precision form."""

from __future__ import annotations

import numpy as np

from oracle import stencils as ora
from stencil_benchmarks_gb300 import array as sbarray
from stencil_benchmarks_gb300.device import Field


def host_field(values, storage="float64", layout=(2, 1, 0), alignment=0, halo=(0, 0, 0)):
    """Copy ``values`` (float array of the halo'd shape) into a host array
    with the reference's layout rules; bfloat16 is stored as bit patterns."""
    values = np.asarray(values)
    arr = sbarray.alloc_array(values.shape, storage, layout, alignment, index_to_align=halo)
    if storage == "bfloat16":
        arr[...] = ora.f32_to_bf16_bits(values.astype(np.float32)).reshape(values.shape)
    else:
        arr[...] = values.astype(arr.dtype)
    return arr


def as_compute(host, storage):
    """Values the kernel reads from ``host`` (bf16 widened to f32)."""
    if storage == "bfloat16":
        return ora.bf16_bits_to_f32(np.ascontiguousarray(host)).reshape(host.shape)
    return np.array(host)


def to_device(host, storage, halo):
    f = Field.like_host(host, storage, halo)
    f.upload(host)
    return f


def empty_like_layout(host):
    """A new host array with exactly ``host``'s strides (padding included)."""
    span = int(np.sum((np.array(host.shape) - 1) * np.array(host.strides))) + host.itemsize
    buf = np.zeros(span, dtype=np.uint8)
    return np.ndarray(host.shape, dtype=host.dtype, buffer=buf, strides=host.strides)


def download_like(field, host):
    out = empty_like_layout(host)
    field.download(out)
    return out


def interior(a, domain, halo):
    return a[ora.inner_slice(domain, halo)]


def round_to_storage(values, storage):
    """Round oracle results (in the compute type) to the storage type."""
    if storage == "bfloat16":
        return ora.f32_to_bf16_bits(np.asarray(values, dtype=np.float32)).reshape(np.shape(values))
    return np.asarray(values).astype(sbarray.storage_numpy_dtype(storage))


def compute_view(host, storage, compute):
    """Halo'd input as the oracle should see it for a (storage, compute) form."""
    vals = as_compute(host, storage)
    return vals.astype(np.float64 if compute == "float64" else np.float32)


def bits_equal(a, b):
    """Bitwise equality, except that any NaN matches any NaN: IEEE 754 leaves
    the sign and payload of a NaN result unspecified, and CPUs and GPUs
    propagate them differently."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape or a.dtype.itemsize != b.dtype.itemsize:
        return False
    view = {8: np.uint64, 4: np.uint32, 2: np.uint16}[a.dtype.itemsize]
    same = a.view(view) == b.view(view)
    if a.dtype.kind == "f":
        same |= np.isnan(a) & np.isnan(b)
    return bool(np.all(same))


def mismatch_report(got, want, limit=5):
    g = np.ascontiguousarray(got)
    w = np.ascontiguousarray(want)
    view = {8: np.uint64, 4: np.uint32, 2: np.uint16}[g.dtype.itemsize]
    differ = g.view(view) != w.view(view)
    if g.dtype.kind == "f":
        differ &= ~(np.isnan(g) & np.isnan(w))
    bad = np.argwhere(differ)
    lines = [f"{len(bad)} of {g.size} differ"]
    for idx in bad[:limit]:
        idx = tuple(idx)
        lines.append(f"  at {idx}: got {g[idx]!r} want {w[idx]!r}")
    return "\n".join(lines)


def rng_fields(seed, shape, names, dists):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = {}
    for n in names:
        lo, hi = dists.get(n, (0.0, 1.0))
        out[n] = rng.uniform(lo, hi, size=shape)
    return out


VADV_DISTS = {
    "ustage": (-1.0, 1.0), "upos": (-1.0, 1.0), "utens": (-1.0, 1.0), "utensstage": (-1.0, 1.0),
    "wcon": (-0.5, 0.5),
}
VADV_ARGS = ("ustage", "upos", "utens", "utensstage", "wcon")
