"""The server on the GPU: generated inputs are reproducible, every served
result equals the oracle, and a request gives the same bits alone and in a
mix of concurrent requests of other sizes and precisions."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from stencil_benchmarks_gb300 import _native, serving
from stencil_benchmarks_gb300.array import storage_numpy_dtype
from stencil_benchmarks_gb300.device import DeviceBuffer, Stream
from tests.gpu_helpers import bits_equal, mismatch_report
from tests.serving_helpers import download_output, expected_output, fill_values

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["float64", "float32", "bfloat16"])
@pytest.mark.parametrize("lo,hi", [(-0.5, 0.5), (0.0, 1.0), (-1.0, 1.0), (0.25, 1.0), (-3.0, 5.0)])
@pytest.mark.parametrize("offset", [0, 8])
def test_device_fill_matches_host_reproduction(storage, lo, hi, offset, lib):
    """Power-of-two spans from 0 or centred take the exact integer route for
    float64, the others the fp64 formula; an offset of 8 bytes takes the
    element-wise path; 100003 elements leave a ragged end."""
    count = 100_003
    itemsize = storage_numpy_dtype(storage).itemsize
    offset = offset // 8 * itemsize  # keeps the element alignment
    buf = DeviceBuffer(count * 8 + 64)
    scratch = DeviceBuffer(1024)
    desc = serving.SbFillDesc(buf.ptr + offset, count, 0x1234567890ABCDEF, lo, hi, _native.storage_code(storage), 0)
    stream = Stream()
    serving._fill([desc], scratch, stream)
    stream.synchronize()
    host = np.empty(count, dtype=storage_numpy_dtype(storage))
    from stencil_benchmarks_gb300.device import copy_to_host

    copy_to_host(host, buf.ptr + offset)
    want = fill_values(0x1234567890ABCDEF, count, lo, hi, storage)
    assert bits_equal(host, want), mismatch_report(host, want)


def test_fill_many_fields_in_one_launch(lib):
    """Several descriptors of mixed storage and size in one call, from a
    page-locked staging area."""
    from stencil_benchmarks_gb300.device import PinnedBuffer, copy_to_host

    specs = [("float64", 1, 0.0, 1.0), ("float32", 17, -1.0, 1.0), ("bfloat16", 4099, -0.5, 0.5),
             ("float64", 70_001, 0.1, 0.7), ("float32", 0, 0.0, 1.0), ("bfloat16", 33, 0.0, 1.0)]
    bufs = [DeviceBuffer(max(1, n) * 8) for _, n, _, _ in specs]
    descs = [serving.SbFillDesc(b.ptr, n, 1000 + q, lo, hi, _native.storage_code(st), 0)
             for q, (b, (st, n, lo, hi)) in enumerate(zip(bufs, specs))]
    staging = PinnedBuffer(ctypes.sizeof(serving.SbFillDesc) * len(descs))
    scratch = DeviceBuffer(ctypes.sizeof(serving.SbFillDesc) * len(descs))
    stream = Stream()
    serving._fill(descs, scratch, stream, staging.ptr)
    stream.synchronize()
    for q, (b, (st, n, lo, hi)) in enumerate(zip(bufs, specs)):
        host = np.empty(n, dtype=storage_numpy_dtype(st))
        if n:
            copy_to_host(host, b.ptr)
        want = fill_values(1000 + q, n, lo, hi, st)
        assert bits_equal(host, want), f"field {q}: " + mismatch_report(host, want)


def _small_mix(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    forms = ["float64", "float32", "bfloat16"]
    return [serving.Request(rid, ("hdiff", "vadv")[int(rng.integers(0, 2))], int(rng.integers(20, 97)),
                            int(rng.integers(20, 97)), int(rng.integers(2, 41)), forms[int(rng.integers(0, 3))],
                            int(rng.integers(0, 2**62)))
            for rid in range(n)]


def test_served_results_match_the_oracle(lib):
    server = serving.Server(budget_bytes=8e9, max_batch=8, max_nk=48, slots_per_form=2, keep_outputs=True)
    reqs = _small_mix(18, 7)
    for r in reqs:
        server.submit(r)
    server.drain()
    for r in reqs:
        got, want = download_output(r), expected_output(r)
        assert bits_equal(got, want), f"request {r}: " + mismatch_report(got, want)
        server.release(r)


def test_same_result_alone_and_in_a_mix(lib):
    probe = serving.Request(0, "vadv", 77, 45, 33, "float32", 987654321)
    alone_srv = serving.Server(budget_bytes=4e9, max_batch=4, max_nk=48, slots_per_form=1, keep_outputs=True)
    alone_srv.submit(probe)
    alone_srv.drain()
    alone = download_output(probe).copy()

    twin = serving.Request(1000, "vadv", 77, 45, 33, "float32", 987654321)
    others = _small_mix(40, 8)
    mixed = others[:20] + [twin] + others[20:]
    srv = serving.Server(budget_bytes=8e9, max_batch=6, max_nk=48, slots_per_form=3, keep_outputs=True)
    for r in mixed:
        srv.submit(r)
        srv.step()  # arrivals interleave with execution
    srv.drain()
    in_mix = download_output(twin)
    assert bits_equal(alone, in_mix), mismatch_report(alone, in_mix)
    assert bits_equal(in_mix, expected_output(twin))


def test_budget_bounded_load(lib):
    reqs = _small_mix(60, 9)
    biggest = max(r.footprint() for r in reqs)
    srv = serving.Server(budget_bytes=2 * biggest, max_batch=4, max_nk=48, slots_per_form=2)
    stats = serving.run_load(srv, reqs, rate=5000.0)
    assert stats["requests"] == 60 and all(r.completed for r in reqs)
    assert srv.pool.peak <= srv.pool.budget
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    assert srv.pool.in_use == 0


def test_fast_float64_serving_within_tolerance(lib):
    """float64 requests served with fixed-point hdiff and float-pair vadv:
    within 1e-12 (hdiff) / 1e-10 (vadv) of the field scale of the oracle,
    and the same bits alone and in a mix."""
    reqs = [r for r in _small_mix(30, 10) if r.storage == "float64"]
    assert reqs
    srv = serving.Server(budget_bytes=8e9, max_batch=6, max_nk=48, slots_per_form=2, keep_outputs=True,
                         float64_compute="fixed64")
    for r in reqs:
        srv.submit(r)
    srv.drain()
    for r in reqs:
        got, want = download_output(r), expected_output(r)
        scale = float(np.max(np.abs(want)))
        tol = 1e-12 if r.op == "hdiff" else 1e-10
        assert float(np.max(np.abs(got - want))) <= tol * scale, r
    probe = reqs[0]
    twin = serving.Request(999, probe.op, probe.ni, probe.nj, probe.nk, "float64", probe.seed)
    alone = serving.Server(budget_bytes=4e9, max_batch=4, max_nk=48, slots_per_form=1, keep_outputs=True,
                           float64_compute="fixed64")
    alone.submit(twin)
    alone.drain()
    assert bits_equal(download_output(twin), download_output(probe))


def test_plain_mode_serves_the_same_bits(lib):
    """mode="plain" (one kernel launch per request, the baseline of the
    batched server) gives every request the oracle's result too."""
    reqs = _small_mix(16, 12)
    srv = serving.Server(budget_bytes=8e9, max_batch=6, max_nk=48, slots_per_form=2, keep_outputs=True, mode="plain")
    stats = serving.run_load(srv, reqs, rate=20000.0)
    assert stats["requests"] == 16 and 0.0 <= stats["host_step_fraction"] <= 1.0
    assert set(stats["by_precision"]) <= {"float64", "float32", "bfloat16"}
    for r in reqs:
        got, want = download_output(r), expected_output(r)
        assert bits_equal(got, want), f"request {r}: " + mismatch_report(got, want)
        srv.release(r)
