"""Bounded device-side waits: a TMA hdiff launch whose plane waits give up
reports SB_ERR_TIMEOUT through the library's status checks, and the status is
cleared once reported.

The give-up is made to happen with the testing aid ``sb_debug_wait_limit(0)``
(every first wait gives up at once).  Nothing faults or hangs: each thread
block then stores nothing for that plane, drains its tensor copies in flight
with the default bound (they land within microseconds) and returns."""

from __future__ import annotations

import ctypes
import time

import numpy as np
import pytest

from oracle import stencils as ora
from stencil_benchmarks_gb300 import _native, kernels
from stencil_benchmarks_gb300.device import Event
from tests.gpu_helpers import bits_equal, download_like, host_field, interior, to_device

pytestmark = pytest.mark.gpu

DOMAIN, HALO = (96, 40, 6), (2, 2, 0)


def _fields(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = tuple(d + 2 * h for d, h in zip(DOMAIN, HALO))
    hosts = {n: host_field(rng.uniform(0.0, 1.0, size=shape), alignment=64, halo=HALO)
             for n in ("inp", "coeff", "out")}
    return hosts, {n: to_device(h, "float64", HALO) for n, h in hosts.items()}


def _launch(dev, timed):
    inp, coeff, out = dev["inp"], dev["coeff"], dev["out"]
    t = ctypes.c_double(0.0)
    tune = _native.tune(variant=_native.HDIFF_TMA)
    return _native.lib().sb_hdiff(0, 0, ctypes.c_void_p(inp.interior_ptr), ctypes.c_void_p(coeff.interior_ptr),
                                  ctypes.c_void_p(out.interior_ptr), *DOMAIN, *inp.strides, ctypes.byref(tune),
                                  None, ctypes.byref(t) if timed else None)


@pytest.fixture
def give_up_at_once(lib):
    _native.call("sb_debug_wait_limit", 0)
    yield
    _native.call("sb_debug_wait_limit", -1)
    _native.lib().sb_synchronize()
    _native.lib().sb_kernel_status()


def test_untimed_give_up_is_reported_by_synchronize(give_up_at_once):
    lib = _native.lib()
    _, dev = _fields(1)
    assert _launch(dev, timed=False) == _native.SB_OK
    assert lib.sb_synchronize() == _native.SB_ERR_TIMEOUT
    assert "gave up" in _native.last_error()
    assert lib.sb_kernel_status() == _native.SB_OK  # cleared by the report


def test_timed_give_up_is_reported_by_the_call(give_up_at_once):
    _, dev = _fields(2)
    assert _launch(dev, timed=True) == _native.SB_ERR_TIMEOUT
    assert _native.lib().sb_kernel_status() == _native.SB_OK


def test_next_hdiff_call_reports_an_earlier_give_up(give_up_at_once):
    lib = _native.lib()
    _, dev = _fields(3)
    done = Event()
    assert _launch(dev, timed=False) == _native.SB_OK
    done.record()
    deadline = time.monotonic() + 30.0
    while lib.sb_event_query(ctypes.c_void_p(done.handle)) != _native.SB_OK:  # no status check on this path
        assert time.monotonic() < deadline, "launch did not complete"
    _native.call("sb_debug_wait_limit", -1)
    assert _launch(dev, timed=False) == _native.SB_ERR_TIMEOUT  # reported before launching anything
    assert _launch(dev, timed=False) == _native.SB_OK
    assert lib.sb_synchronize() == _native.SB_OK


def test_after_a_give_up_the_default_limit_computes_exactly(lib):
    _native.call("sb_debug_wait_limit", 0)
    hosts, dev = _fields(4)
    try:
        assert _launch(dev, timed=True) == _native.SB_ERR_TIMEOUT
    finally:
        _native.call("sb_debug_wait_limit", -1)
    kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], tune=_native.tune(variant=_native.HDIFF_TMA))
    _native.synchronize()
    got = interior(download_like(dev["out"], hosts["out"]), DOMAIN, HALO)
    want = ora.hdiff(np.array(hosts["inp"]), np.array(hosts["coeff"]), DOMAIN, HALO)
    assert bits_equal(got, want)
