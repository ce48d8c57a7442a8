"""sb_vadv_noalloc: vertical advection that allocates no device memory.

Some callers cannot call cudaMalloc -- for instance code embedded in a host
framework that owns every device allocation through fixed memory pools, or
that must avoid the device-wide synchronisation cudaMalloc/cudaFree can
cause.  sb_vadv_noalloc keeps the elimination factors in a fixed array inside
the library instead of caller-provided scratch.  These tests call it through
the C ABI and check that two calls in a row give exactly what the regular
entry point sb_vadv gives (bit-identical, the tolerance of every fp64 and
fp32 parity test here), and exactly what the oracle computes in the compute
type on the stored inputs, rounded once to storage.  The file is named so
that pytest collects it last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, kernels
from tests.gpu_helpers import (
    VADV_ARGS,
    VADV_DISTS,
    bits_equal,
    compute_view,
    download_like,
    host_field,
    interior,
    mismatch_report,
    rng_fields,
    round_to_storage,
    to_device,
)

pytestmark = pytest.mark.gpu


def _fields(domain, halo, storage, seed):
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    vals = rng_fields(seed, shape, VADV_ARGS, VADV_DISTS)
    vals["out"] = np.zeros(shape)
    hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
    dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
    return hosts, dev


def _noalloc(dev, domain, storage, compute, shift=(1, 0)):
    f = dev["ustage"]
    args = [
        _native.storage_code(storage), _native.storage_code(compute),
        *(ctypes.c_void_p(dev[n].interior_ptr) for n in ("ustage", "upos", "utens", "utensstage", "wcon", "out")),
        *domain, *f.strides, shift[0], shift[1], None, None,
    ]
    rc = _native.lib().sb_vadv_noalloc(*args)
    if rc != _native.SB_OK:
        raise _native.SbError("sb_vadv_noalloc", rc, _native.last_error())


@pytest.mark.parametrize("storage,compute", [("float64", "float64"), ("float32", "float32"), ("float32", "float64"),
                                             ("bfloat16", "float32")])
def test_noalloc_matches_regular_entry_point_twice(storage, compute, lib):
    # two calls in a row on different problems: the second must not see
    # anything the first left in the shared scratch array
    for call, (domain, seed, shift) in enumerate([((70, 31, 40), 1, (1, 0)), ((45, 52, 17), 2, (0, 1))]):
        halo = (1, 1, 0)
        hosts, dev = _fields(domain, halo, storage, seed)
        _noalloc(dev, domain, storage, compute, shift)
        _native.synchronize()
        got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
        kernels.vadv(dev["ustage"], dev["upos"], dev["utens"], dev["utensstage"], dev["wcon"], shift,
                     out=dev["utensstage"], compute=compute)
        want = interior(download_like(dev["utensstage"], hosts["utensstage"]), domain, halo)
        assert bits_equal(got, want), f"call {call}: " + mismatch_report(got, want)
        oracle = ora._vadv_component(*(compute_view(hosts[n], storage, compute) for n in VADV_ARGS),
                                     domain, halo, *shift)
        want = round_to_storage(oracle, storage)
        assert bits_equal(got, want), f"call {call} vs the oracle: " + mismatch_report(got, want)


def test_noalloc_rejects_columns_taller_than_its_scratch(lib):
    # 32 MiB / (2 * 8 bytes * 64 slots) = 32768 levels fit; ask for more
    domain, halo = (4, 2, 40000), (1, 0, 0)
    f = ctypes.c_void_p(8)  # never dereferenced: the size check fails first
    rc = _native.lib().sb_vadv_noalloc(_native.SB_F64, _native.SB_F64, f, f, f, f, f, f, *domain,
                                       1, 6, 12, 1, 0, None, None)
    assert rc == _native.SB_ERR_BUDGET
    assert "static scratch array" in _native.last_error()
