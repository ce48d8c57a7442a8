"""Parity at the benchmark workloads' own sizes, against the oracle.

* hdiff fp64 on 128x128x64 with a (2, 2, 0) halo (arrays 132x132x64): every
  hdiff variant bit for bit, with the L2 flushed before each launch;
* the 64 uneven float32 domains (32 hdiff + 32 vadv, ni, nj in {32..512},
  nk in [40, 137], seed 3) in one autotuned batched launch: every domain bit
  for bit (the C oracle, same bits as the numpy oracle);
* a sample of the serving workload (ni, nj log-uniform to 1024, nk to 137,
  fp64 / fp32 / bf16-storage requests, plus the largest 1024 x 1024 x 137
  and 1024 x 1024 x 40 requests), served with continuous batching under
  Poisson arrivals: every request bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import cport
from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, autotune, kernels, serving
from stencil_benchmarks_gb300.batching import Batch
from stencil_benchmarks_gb300.device import l2_flush
from stencil_benchmarks_gb300.workloads import device_domain, uneven_specs
from tests.gpu_helpers import bits_equal, download_like, host_field, interior, mismatch_report, to_device
from tests.serving_helpers import download_output, expected_output_c

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [_native.HDIFF_TMA, _native.HDIFF_TILE, _native.HDIFF_JSCAN,
                                     _native.HDIFF_VSCAN])
@pytest.mark.parametrize("alignment", [0, 64])
def test_hdiff_fp64_128x128x64(variant, alignment, lib):
    domain, halo = (128, 128, 64), (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(128))
    hosts = {n: host_field(rng.uniform(0.0, 1.0, size=shape), alignment=alignment, halo=halo)
             for n in ("inp", "coeff", "out")}
    assert hosts["inp"].shape == (132, 132, 64)
    dev = {n: to_device(h, "float64", halo) for n, h in hosts.items()}
    want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), domain, halo)
    for _ in range(2):
        l2_flush()
        kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], tune=_native.tune(variant=variant))
        _native.synchronize()
        got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
        assert bits_equal(got, want), mismatch_report(got, want)


def test_uneven_64_domain_batch_matches_the_oracle(lib):
    specs = uneven_specs(seed=3, n=64)
    built = [device_domain(s, "float32") for s in specs]
    doms, devs, hosts = zip(*built)
    max_nk = max(s.nk for s in specs)
    best, _ = autotune.autotune_batch("float32", doms, max_nk)
    batch = Batch("float32", max_domains=64, max_nk=max_nk, **best)
    batch.set(doms)
    for _ in range(2):  # the capture and a replay of the graph
        batch.launch()
        _native.synchronize()
    for q, (spec, dev, host) in enumerate(zip(specs, devs, hosts)):
        domain = (spec.ni, spec.nj, spec.nk)
        halo = dev["out"].halo
        got = interior(download_like(dev["out"], host["out"]), domain, halo)
        out = np.zeros_like(host["out"])
        if spec.op == "hdiff":
            cport.hdiff(host["inp"], host["coeff"], out, domain, halo)
        else:
            cport.vadv(host["stage"], host["pos"], host["tens"], host["tensstage"], host["wcon"], domain, halo,
                       (1, 0), out=out)
        want = interior(out, domain, halo)
        assert bits_equal(got, want), f"domain {q} {spec}: " + mismatch_report(got, want)


def test_serving_workload_sample_matches_the_oracle(lib):
    reqs = serving.request_specs(24, seed=13)
    reqs += [serving.Request(100, "vadv", 1024, 1024, 137, "float64", 77),
             serving.Request(101, "hdiff", 1024, 1024, 40, "bfloat16", 78),
             serving.Request(102, "vadv", 1024, 992, 137, "float32", 79)]
    assert {r.storage for r in reqs} == {"float64", "float32", "bfloat16"}
    server = serving.Server(budget_bytes=24e9, max_batch=16, slots_per_form=3, keep_outputs=True)
    stats = serving.run_load(server, reqs, rate=2000.0)
    assert stats["requests"] == len(reqs)
    for r in reqs:
        got, want = download_output(r), expected_output_c(r)
        assert bits_equal(got, want), f"request {r.rid} {r.op} {r.ni}x{r.nj}x{r.nk} {r.storage}: " + \
            mismatch_report(got, want)
        server.release(r)
