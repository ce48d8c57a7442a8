"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations.

* single domain, 512 x 512 x 80: hdiff fields U[0, 1); vadv stage/pos/tens/
  tensstage U[-1, 1), wcon U[-0.5, 0.5), dtr_stage = 3/20 (built into the
  kernels);
* batched uneven domains: ``uneven_specs(seed, n)`` draws ni, nj uniformly
  from {32, 64, ..., 512} and nk uniformly from {40, ..., 137}, half hdiff and
  half vadv, from one seed;
* serving requests: ``request_specs`` (log-uniform ni, nj in [32, 1024]
  rounded to a multiple of 32, nk uniform in [40, 137], precision fp64 / fp32
  / bf16-storage at 20 / 60 / 20 %, Poisson arrivals).

Fields use the reference's layout (i unit-stride, halo 2 in i/j for hdiff,
1 in i/j for vadv) and are created directly on the device from host arrays.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import array as sbarray
from .batching import HdiffDomain, VadvDomain
from .device import Field

HDIFF_HALO = (2, 2, 0)
VADV_HALO = (1, 1, 0)


@dataclass
class DomainSpec:
    op: str  # "hdiff" or "vadv"
    ni: int
    nj: int
    nk: int
    seed: int

    @property
    def points(self) -> int:
        return self.ni * self.nj * self.nk

    def compulsory_bytes(self, itemsize: int) -> int:
        if self.op == "hdiff":
            return itemsize * ((self.ni + 4) * (self.nj + 4) * self.nk + 2 * self.points)
        return itemsize * (5 * self.points + (self.ni + 1) * self.nj * self.nk)


def uneven_specs(seed: int = 3, n: int = 64):
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.arange(32, 513, 32)
    specs = []
    for q in range(n):
        op = "hdiff" if q % 2 == 0 else "vadv"
        ni, nj = (int(x) for x in rng.choice(sizes, size=2))
        nk = int(rng.integers(40, 138))
        specs.append(DomainSpec(op, ni, nj, nk, int(rng.integers(0, 2**31))))
    return specs


def host_fields(spec: DomainSpec, storage: str):
    """Seeded host arrays (reference layout) for one domain: name -> array."""
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    halo = HDIFF_HALO if spec.op == "hdiff" else VADV_HALO
    shape = (spec.ni + 2 * halo[0], spec.nj + 2 * halo[1], spec.nk + 2 * halo[2])
    if spec.op == "hdiff":
        dists = {"inp": (0.0, 1.0), "coeff": (0.0, 1.0), "out": (0.0, 0.0)}
    else:
        dists = {"stage": (-1.0, 1.0), "pos": (-1.0, 1.0), "tens": (-1.0, 1.0), "tensstage": (-1.0, 1.0),
                 "wcon": (-0.5, 0.5), "out": (0.0, 0.0)}
    out = {}
    for name, (lo, hi) in dists.items():
        a = sbarray.alloc_array(shape, storage, (2, 1, 0), 0, index_to_align=halo)
        vals = rng.uniform(lo, hi, size=shape) if hi > lo else np.zeros(shape)
        if storage == "bfloat16":
            bits = vals.astype(np.float32).view(np.uint32).astype(np.uint64)
            a[...] = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
        else:
            a[...] = vals
        out[name] = a
    return out, halo


def device_domain(spec: DomainSpec, storage: str, hosts=None):
    """Upload one domain; returns (batch domain, {name: Field}, {name: host array})."""
    if hosts is None:
        hosts, halo = host_fields(spec, storage)
    else:
        halo = HDIFF_HALO if spec.op == "hdiff" else VADV_HALO
    dev = {n: Field.like_host(h, storage, halo) for n, h in hosts.items()}
    for n, h in hosts.items():
        dev[n].upload(h)
    if spec.op == "hdiff":
        dom = HdiffDomain(dev["inp"], dev["coeff"], dev["out"])
    else:
        dom = VadvDomain(dev["stage"], dev["pos"], dev["tens"], dev["tensstage"], dev["wcon"], out=dev["out"])
    return dom, dev, hosts
