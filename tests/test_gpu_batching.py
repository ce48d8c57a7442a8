"""The persistent batched kernel gives exactly the per-domain results."""

from __future__ import annotations

import numpy as np
import pytest

from stencil_benchmarks_gb300 import _native, kernels
from stencil_benchmarks_gb300.batching import Batch
from stencil_benchmarks_gb300.workloads import DomainSpec, device_domain
from tests.gpu_helpers import bits_equal, download_like, mismatch_report

pytestmark = pytest.mark.gpu

FORMS = [("float64", "float64"), ("float32", "float32"), ("bfloat16", "float32"), ("float32", "float64")]


def _random_specs(seed, n, max_ij=160, max_k=40):
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for q in range(n):
        op = ("hdiff", "vadv")[int(rng.integers(0, 2))]
        ni, nj = (int(x) for x in rng.integers(1, max_ij + 1, size=2))
        nk = int(rng.integers(2, max_k + 1))
        specs.append(DomainSpec(op, ni, nj, nk, int(rng.integers(0, 2**31))))
    return specs


def _reference_outputs(specs, doms, devs, hosts, compute):
    """Per-domain launches of the plain kernels into fresh output fields."""
    refs = []
    for spec, dom, dev, host in zip(specs, doms, devs, hosts):
        from stencil_benchmarks_gb300.device import Field

        out = Field.like_host(host["out"], dev["out"].storage, dev["out"].halo)
        if spec.op == "hdiff":
            kernels.hdiff(dom.inp, dom.coeff, out, compute=compute)
        else:
            kernels.vadv(dom.stage, dom.pos, dom.tens, dom.tensstage, dom.wcon, out=out, compute=compute)
        refs.append(out)
    _native.synchronize()
    return refs


def _check(specs, devs, hosts, refs):
    # interiors only: the reference outputs are fresh allocations whose halo
    # holds whatever the allocator's memory held before
    for q, (spec, dev, host, ref) in enumerate(zip(specs, devs, hosts, refs)):
        halo = dev["out"].halo
        sl = tuple(slice(h, h + n) for h, n in zip(halo, (spec.ni, spec.nj, spec.nk)))
        got = download_like(dev["out"], host["out"])[sl]
        want = download_like(ref, host["out"])[sl]
        assert bits_equal(got, want), f"domain {q} {spec}: " + mismatch_report(got, want)


@pytest.mark.parametrize("storage,compute", FORMS)
def test_batch_matches_per_domain_kernels(storage, compute, lib):
    specs = _random_specs(11, 20)
    built = [device_domain(s, storage) for s in specs]
    doms, devs, hosts = zip(*built)
    refs = _reference_outputs(specs, doms, devs, hosts, compute)
    batch = Batch(storage, compute, max_domains=32, max_nk=64)
    batch.set(doms)
    batch.launch()
    _native.synchronize()
    _check(specs, devs, hosts, refs)
    assert batch.info()["items"] > 0


@pytest.mark.parametrize("block,per_sm,rows,planes,order", [(32, 1, 1, 1, 0), (64, 2, 7, 3, 1), (128, 4, 32, 1, 0),
                                                            (256, 8, 64, 2, 1), (96, 3, 16, 5, 0)])
def test_batch_tunings(block, per_sm, rows, planes, order, lib):
    specs = _random_specs(12, 12, max_ij=100, max_k=30)
    built = [device_domain(s, "float32") for s in specs]
    doms, devs, hosts = zip(*built)
    refs = _reference_outputs(specs, doms, devs, hosts, "float32")
    batch = Batch("float32", max_domains=16, max_nk=32, block=block, blocks_per_sm=per_sm, hdiff_rows=rows,
                  hdiff_planes=planes, order=order)
    batch.set(doms)
    batch.launch()
    _native.synchronize()
    _check(specs, devs, hosts, refs)


@pytest.mark.parametrize("storage", ["float32", "bfloat16"])
@pytest.mark.parametrize("vadv_block,max_nk", [(32, 256), (64, 256), (32, 300)])
def test_batch_vadv_paths(storage, vadv_block, max_nk, lib):
    """float32 vadv with the factors in tensor memory (vadv block 32, nk <= 256;
    each bucket's blocks sized for its cap) and the shared-memory / slab path
    (vadv block 64, or max_nk above 256) give the per-domain results."""
    specs = _random_specs(31, 10, max_ij=70, max_k=256)
    built = [device_domain(s, storage) for s in specs]
    doms, devs, hosts = zip(*built)
    refs = _reference_outputs(specs, doms, devs, hosts, "float32")
    batch = Batch(storage, "float32", max_domains=16, max_nk=max_nk, vadv_block=vadv_block)
    for _ in range(2):  # the second replay reuses the captured graph
        batch.set(doms)
        batch.launch()
        _native.synchronize()
        _check(specs, devs, hosts, refs)


def test_batch_reuse_replays_the_graph_with_a_new_table(lib):
    batch = Batch("float32", max_domains=16, max_nk=48)
    for seed in (21, 22, 23):
        specs = _random_specs(seed, 9, max_ij=90, max_k=48)
        built = [device_domain(s, "float32") for s in specs]
        doms, devs, hosts = zip(*built)
        refs = _reference_outputs(specs, doms, devs, hosts, "float32")
        batch.set(doms)
        t = batch.launch(timed=True)
        assert t > 0
        _check(specs, devs, hosts, refs)


def test_empty_batch_and_in_place_vadv(lib):
    batch = Batch("float64", max_domains=4, max_nk=16)
    batch.set([])
    batch.launch()
    spec = DomainSpec("vadv", 40, 7, 12, 5)
    dom, dev, host = device_domain(spec, "float64")
    ref = _reference_outputs([spec], [dom], [dev], [host], "float64")[0]
    dom.out = None  # in place: the new tensstage overwrites tensstage
    batch.set([dom])
    batch.launch()
    _native.synchronize()
    sl = (slice(1, 41), slice(1, 8), slice(0, 12))
    got = download_like(dev["tensstage"], host["tensstage"])[sl]
    want = download_like(ref, host["out"])[sl]
    assert bits_equal(got, want)


def test_batch_rejects_bad_domains(lib):
    batch = Batch("float32", max_domains=2, max_nk=8)
    spec = DomainSpec("vadv", 8, 4, 9, 1)
    dom, _, _ = device_domain(spec, "float32")
    with pytest.raises(_native.SbError, match="max_nk"):
        batch.set([dom])
    small = device_domain(DomainSpec("hdiff", 8, 4, 3, 2), "float32")[0]
    with pytest.raises(_native.SbError, match="capacity"):
        batch.set([small, small, small])
    one_level = device_domain(DomainSpec("vadv", 8, 4, 1, 3), "float32")[0]
    with pytest.raises(_native.SbError, match="nk >= 2"):
        batch.set([one_level])
