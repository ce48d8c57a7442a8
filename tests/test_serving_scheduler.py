"""Scheduling logic of the server on the CPU: admission by memory budget in
arrival order, continuous batching over several in-flight slots, pool reuse.
The device is replaced by fakes (no GPU work happens here)."""

from __future__ import annotations

import itertools

import numpy as np
import pytest

from stencil_benchmarks_gb300 import serving


class FakeBuffer:
    _ptrs = itertools.count(1 << 20, 1 << 20)

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        self.ptr = next(FakeBuffer._ptrs)
        self.freed = False

    def free(self):
        self.freed = True


class FakeBatch:
    launches = []

    def __init__(self, storage, compute, max_domains, max_nk, **kw):
        self.storage, self.max_domains = storage, max_domains
        self.domains = []

    def set(self, domains):
        assert len(domains) <= self.max_domains
        self.domains = list(domains)

    def launch(self, stream=None, timed=False):
        FakeBatch.launches.append((self.storage, len(self.domains)))


class FakeHandle:
    def __init__(self):
        self.handle = id(self)
        self.as_parameter = None

    def record(self, stream=None):
        pass


@pytest.fixture
def fake_device(monkeypatch):
    done = set()
    monkeypatch.setattr(serving, "DeviceBuffer", FakeBuffer)
    monkeypatch.setattr(serving, "Batch", FakeBatch)
    monkeypatch.setattr(serving, "Stream", FakeHandle)
    monkeypatch.setattr(serving, "Event", FakeHandle)
    monkeypatch.setattr(serving, "_fill", lambda descs, scratch, stream: None)
    monkeypatch.setattr(serving, "_wait", lambda stream, event: None)
    monkeypatch.setattr(serving, "_event_done", lambda ev: id(ev) in done)
    monkeypatch.setattr(serving._native, "call", lambda *a, **k: 0)
    FakeBatch.launches = []
    return done


def _req(rid, op="hdiff", n=64, nk=10, storage="float32"):
    return serving.Request(rid, op, n, n, nk, storage, seed=rid)


def _complete_all(server, done):
    for slots in server.slots.values():
        for s in slots:
            if s.busy:
                done.add(id(s.done))


def test_admission_respects_budget_in_arrival_order(fake_device):
    one = _req(0).footprint()
    server = serving.Server(budget_bytes=2 * one, max_batch=8, slots_per_form=2)
    reqs = [_req(i) for i in range(5)]
    for r in reqs:
        server.submit(r)
    server.step()
    assert [r.admitted is not None for r in reqs] == [True, True, False, False, False]
    assert server.pool.in_use <= server.pool.budget
    _complete_all(server, fake_device)
    server.step()  # retire 0, 1; admit 2, 3
    assert reqs[0].completed and reqs[1].completed
    assert [r.admitted is not None for r in reqs] == [True] * 4 + [False]
    while server.busy():
        _complete_all(server, fake_device)
        server.step()
    assert all(r.completed for r in reqs)
    assert server.pool.peak <= server.pool.budget
    assert server.pool.in_use == 0


def test_continuous_batching_overlaps_slots(fake_device):
    server = serving.Server(budget_bytes=1e12, max_batch=4, slots_per_form=3)
    first = [_req(i) for i in range(4)]
    for r in first:
        server.submit(r)
    server.step()
    assert FakeBatch.launches == [("float32", 4)]
    # new arrivals while the first batch still runs go out in a second slot
    late = [_req(10 + i) for i in range(3)]
    for r in late:
        server.submit(r)
    server.step()
    assert FakeBatch.launches == [("float32", 4), ("float32", 3)]
    busy = sum(s.busy for s in server.slots["float32"])
    assert busy == 2
    _complete_all(server, fake_device)
    server.step()
    assert all(r.completed for r in first + late)


def test_forms_go_to_their_own_batches(fake_device):
    server = serving.Server(budget_bytes=1e12, max_batch=8, slots_per_form=1)
    for i, st in enumerate(["float64", "float32", "bfloat16", "float32"]):
        server.submit(_req(i, op="vadv" if i % 2 else "hdiff", storage=st))
    server.step()
    assert sorted(FakeBatch.launches) == [("bfloat16", 1), ("float32", 2), ("float64", 1)]


def test_slots_limit_in_flight_batches(fake_device):
    server = serving.Server(budget_bytes=1e12, max_batch=2, slots_per_form=2)
    reqs = [_req(i) for i in range(9)]
    for r in reqs:
        server.submit(r)
    server.step()
    assert len(FakeBatch.launches) == 2  # two slots, two requests each
    assert len(server.ready["float32"]) == 5
    while server.busy():
        _complete_all(server, fake_device)
        server.step()
    assert sum(n for _, n in FakeBatch.launches) == 9


def test_pool_reuses_size_classes_and_evicts_cached(fake_device):
    pool = serving.DevicePool(budget_bytes=10 * serving.GRANULE)
    a = pool.try_alloc(3 * serving.GRANULE - 5)
    assert a.nbytes == 3 * serving.GRANULE
    pool.release(a)
    b = pool.try_alloc(3 * serving.GRANULE)
    assert b is a  # same size class: reused
    c = pool.try_alloc(6 * serving.GRANULE)
    assert c is not None and pool.in_use == 9 * serving.GRANULE
    assert pool.try_alloc(2 * serving.GRANULE) is None  # over budget
    pool.release(c)
    d = pool.try_alloc(5 * serving.GRANULE)  # evicts the cached 6-granule buffer
    assert d is not None and c.freed
    assert pool.in_use + pool.cached <= pool.budget


def test_invalid_requests_rejected(fake_device):
    server = serving.Server(budget_bytes=1e9, max_nk=50)
    with pytest.raises(ValueError):
        server.submit(_req(0, storage="float16"))
    with pytest.raises(ValueError):
        server.submit(_req(1, op="vadv", nk=51))
    with pytest.raises(ValueError):
        server.submit(_req(2, n=4096, nk=100))  # larger than the budget


def test_keep_outputs_and_release(fake_device):
    server = serving.Server(budget_bytes=1e12, keep_outputs=True)
    r = _req(0)
    server.submit(r)
    server.step()
    _complete_all(server, fake_device)
    server.step()
    assert set(r.fields) == {"out"}
    before = server.pool.in_use
    server.release(r)
    assert server.pool.in_use < before and not r.fields


def test_request_specs_distribution():
    reqs = serving.request_specs(4000, seed=3)
    sizes = np.array([[r.ni, r.nj] for r in reqs])
    assert sizes.min() >= 32 and sizes.max() <= 1024 and np.all(sizes % 32 == 0)
    nks = np.array([r.nk for r in reqs])
    assert nks.min() >= 40 and nks.max() <= 137
    frac = {s: np.mean([r.storage == s for r in reqs]) for s in serving.FORMS}
    assert abs(frac["float64"] - 0.2) < 0.03 and abs(frac["float32"] - 0.6) < 0.03
    assert abs(np.mean([r.op == "hdiff" for r in reqs]) - 0.5) < 0.03
    # log-uniform: the median size is near the geometric mean of 32 and 1024
    assert 120 < np.median(sizes) < 260
