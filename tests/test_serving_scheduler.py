"""Scheduling logic of the native server on the CPU: admission by memory
budget in arrival order, continuous batching over several in-flight slots,
forms, kept fields.  The server runs in its simulating mode (no CUDA call:
launches are recorded, in-flight work completes on request), so no GPU work
happens here; the arena tests use a fake device region."""

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


@pytest.fixture(scope="module", autouse=True)
def _library_built():
    """The scheduler and the arena are host code in the native library (no GPU needed)."""
    from stencil_benchmarks_gb300 import build

    build.build()


@pytest.fixture
def fake_region(monkeypatch):
    monkeypatch.setattr(serving, "DeviceBuffer", FakeBuffer)


def _req(rid, op="hdiff", n=64, nk=10, storage="float32"):
    return serving.Request(rid, op, n, n, nk, storage, seed=rid)


def _server(**kw):
    return serving.Server(simulate=True, **kw)


def _run_out(server):
    while server.step():
        server.debug_complete()


def test_admission_respects_budget_in_arrival_order():
    one = _req(0).footprint()
    server = _server(budget_bytes=2 * one, max_batch=8, slots_per_form=2)
    reqs = [_req(i) for i in range(5)]
    for r in reqs:
        server.submit(r)
    server.step()
    assert [server.query(r).admitted is not None for r in reqs] == [True, True, False, False, False]
    assert server.pool.in_use <= server.pool.budget
    server.debug_complete()
    server.step()  # retire 0, 1; admit 2, 3
    assert reqs[0].completed and reqs[1].completed
    assert [server.query(r).admitted is not None for r in reqs] == [True] * 4 + [False]
    _run_out(server)
    assert all(r.completed for r in reqs) and len(server.completed) == 5
    assert all(r.arrival <= r.admitted <= r.launched <= r.completed for r in reqs)
    assert server.pool.peak <= server.pool.budget
    assert server.pool.in_use == 0


def test_continuous_batching_overlaps_slots():
    server = _server(budget_bytes=1e12, max_batch=4, slots_per_form=3)
    first = [_req(i) for i in range(4)]
    for r in first:
        server.submit(r)
    server.step()
    assert server.launches() == [("float32", 4)]
    # new arrivals while the first batch still runs go out in a second slot
    late = [_req(10 + i) for i in range(3)]
    for r in late:
        server.submit(r)
    server.step()
    assert server.launches() == [("float32", 4), ("float32", 3)]
    assert server.state().busy_slots == 2
    server.debug_complete()
    server.step()
    assert all(r.completed for r in first + late)


def test_forms_go_to_their_own_batches():
    server = _server(budget_bytes=1e12, max_batch=8, slots_per_form=1)
    for i, st in enumerate(["float64", "float32", "bfloat16", "float32"]):
        server.submit(_req(i, op="vadv" if i % 2 else "hdiff", storage=st))
    server.step()
    assert sorted(server.launches()) == [("bfloat16", 1), ("float32", 2), ("float64", 1)]


def test_slots_limit_in_flight_batches():
    server = _server(budget_bytes=1e12, max_batch=2, slots_per_form=2)
    reqs = [_req(i) for i in range(9)]
    for r in reqs:
        server.submit(r)
    server.step()
    assert len(server.launches()) == 2  # two slots, two requests each
    assert server.state().ready == 5
    _run_out(server)
    assert sum(n for _, n in server.launches()) == 9 and all(r.completed for r in reqs)


def test_many_requests_under_a_tight_budget_all_complete():
    rng = np.random.Generator(np.random.PCG64(5))
    reqs = [_req(i, op=("hdiff", "vadv")[i % 2], n=int(rng.integers(8, 200)), nk=int(rng.integers(2, 60)),
                 storage=("float64", "float32", "bfloat16")[i % 3]) for i in range(300)]
    budget = 3 * max(r.footprint() for r in reqs)
    server = _server(budget_bytes=budget, max_batch=5, slots_per_form=2, max_nk=60)
    for r in reqs[:150]:
        server.submit(r)
    server.step()
    for r in reqs[150:]:
        server.submit(r)
    _run_out(server)
    assert len(server.completed) == 300 and server.pool.in_use == 0
    assert server.pool.peak <= budget and server.max_waiting >= 150


def test_pool_arena_best_fit_and_coalescing(fake_region):
    A = serving.ALIGN
    pool = serving.DevicePool(budget_bytes=100 * A)
    base = pool.region.ptr
    a = pool.try_alloc(10 * A - 5)
    assert (a.ptr, a.nbytes) == (base, 10 * A)
    b = pool.try_alloc(20 * A)
    c = pool.try_alloc(30 * A)
    d = pool.try_alloc(40 * A)
    assert [x.ptr - base for x in (b, c, d)] == [10 * A, 30 * A, 60 * A]
    assert pool.in_use == 100 * A and pool.try_alloc(1) is None  # budget exhausted
    pool.release(b)
    pool.release(d)
    e = pool.try_alloc(15 * A)  # best fit: the 20-unit hole, not the 40-unit one
    assert e.ptr == base + 10 * A
    pool.release(a)
    pool.release(e)  # coalesces with the freed head: 0..30 is one free piece
    assert pool.stats()["largest_free"] == 40 * A and pool.stats()["free_blocks"] == 2
    pool.release(c)  # everything merges back into one piece
    st = pool.stats()
    assert st == {"in_use": 0, "peak": 100 * A, "largest_free": 100 * A, "free_blocks": 1}
    with pytest.raises(serving._native.SbError):
        pool.release(c)  # double free is an error, not silent corruption


def test_pool_random_churn_keeps_invariants(fake_region):
    A = serving.ALIGN
    pool = serving.DevicePool(budget_bytes=4096 * A)
    base = pool.region.ptr
    rng = np.random.Generator(np.random.PCG64(1))
    live = []
    for _ in range(3000):
        if live and rng.random() < 0.45:
            pool.release(live.pop(int(rng.integers(0, len(live)))))
        else:
            blk = pool.try_alloc(int(rng.integers(1, 200 * A)))
            if blk is not None:
                live.append(blk)
        spans = sorted((x.ptr - base, x.ptr - base + x.nbytes) for x in live)
        assert all(s[1] <= t[0] for s, t in zip(spans, spans[1:]))  # no overlap
        assert all(0 <= s[0] and s[1] <= 4096 * A and s[0] % A == 0 for s in spans)
        assert pool.in_use == sum(x.nbytes for x in live)
    for blk in live:
        pool.release(blk)
    assert pool.stats()["free_blocks"] == 1 and pool.in_use == 0


def test_invalid_requests_rejected():
    server = _server(budget_bytes=1e9, max_nk=50)
    with pytest.raises(ValueError):
        server.submit(_req(0, storage="float16"))
    with pytest.raises(ValueError, match="max_nk"):
        server.submit(_req(1, op="vadv", nk=51))
    with pytest.raises(ValueError, match="budget"):
        server.submit(_req(2, n=4096, nk=100))  # larger than the whole budget


def test_keep_outputs_and_release():
    server = _server(budget_bytes=1e12, keep_outputs=True)
    r = _req(0)
    server.submit(r)
    server.step()
    server.debug_complete()
    server.step()
    assert set(r.fields) == {"out"}
    assert r.fields["out"].shape == (68, 68, 10) and r.fields["out"].strides == (1, 68, 68 * 68)
    before = server.pool.in_use
    server.release(r)
    assert server.pool.in_use < before and not r.fields


def test_keep_inputs_too():
    server = _server(budget_bytes=1e12, keep_outputs=True, keep_inputs=True)
    r = _req(0, op="vadv")
    server.submit(r)
    server.step()
    server.debug_complete()
    server.step()
    assert set(r.fields) == {"stage", "pos", "tens", "tensstage", "wcon", "out"}
    server.release(r)
    assert server.pool.in_use == 0


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


def _f64_exact_route(k, lo, span):
    """The fill kernel's integer construction of lo + span * k * 2^-53 (for a
    power-of-two span with lo = 0 or lo = -span/2), restated on integers."""
    import struct

    P = int(np.log2(span))
    x = k - (1 << 52 if lo != 0.0 else 0)
    if x == 0:
        return 0.0
    sign = 1 << 63 if x < 0 else 0
    a = abs(x)
    msb = a.bit_length() - 1
    mant = (a << (52 - msb)) & ((1 << 52) - 1)
    return struct.unpack("<d", struct.pack("<Q", sign | ((1023 + msb + P - 53) << 52) | mant))[0]


@pytest.mark.parametrize("lo,span", [(0.0, 1.0), (-1.0, 2.0), (-0.5, 1.0), (0.0, 2.0**-40), (-2.0**9, 2.0**10)])
def test_fill_integer_route_equals_fp64_formula(lo, span):
    rng = np.random.Generator(np.random.PCG64(4))
    ks = [0, 1, 2, (1 << 52) - 1, 1 << 52, (1 << 52) + 1, (1 << 53) - 1]
    ks += [int(v) for v in rng.integers(0, 1 << 53, size=3000, dtype=np.int64)]
    for k in ks:
        want = lo + span * (float(k) * 2.0**-53)
        got = _f64_exact_route(k, lo, span)
        assert np.float64(got).tobytes() == np.float64(want).tobytes(), (k, got, want)
