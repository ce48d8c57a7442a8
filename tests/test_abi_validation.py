"""Argument checking of the C ABI, on the CPU: every call below is rejected
(or is a zero-size no-op) before the library touches a device, so no GPU is
needed.  Status codes and messages follow include/sbgb300.h."""

from __future__ import annotations

import ctypes

import pytest

from stencil_benchmarks_gb300 import _native
from stencil_benchmarks_gb300 import build as sbbuild

OK, INVALID, UNSUPPORTED = _native.SB_OK, _native.SB_ERR_INVALID, _native.SB_ERR_UNSUPPORTED
F64, F32, BF16, F32X2, FIX64 = _native.SB_F64, _native.SB_F32, _native.SB_BF16, _native.SB_F32X2, _native.SB_FIX64
P = ctypes.c_void_p(0x1000)  # never dereferenced: every call here stops at its argument checks
NULL = ctypes.c_void_p(0)


@pytest.fixture(scope="module")
def lib():
    sbbuild.build()
    return _native.lib()


def _msg():
    return _native.last_error()


def hdiff(lib, storage, compute, inp=P, ni=8, nj=8, nk=4, strides=(1, 12, 144)):
    t = ctypes.c_double(-1.0)
    rc = lib.sb_hdiff(storage, compute, inp, P, P, ni, nj, nk, *strides, None, None, ctypes.byref(t))
    return rc, t.value


def vadv(lib, storage, compute, nk=4, shift=(1, 0), stage=P):
    return lib.sb_vadv(storage, compute, stage, P, P, P, P, P, None, None, 8, 8, nk, 1, 10, 100, shift[0],
                       shift[1], None, None, None)


def test_hdiff_argument_checks(lib):
    assert hdiff(lib, F64, F64, inp=NULL)[0] == INVALID and "NULL" in _msg()
    assert hdiff(lib, F64, F64, ni=-1)[0] == INVALID and "negative" in _msg()
    assert hdiff(lib, F64, F64, strides=(1, 0, 144))[0] == INVALID and "stride" in _msg()
    assert hdiff(lib, F64, F64, ni=1 << 31)[0] == INVALID
    assert hdiff(lib, BF16, F64)[0] == UNSUPPORTED  # no bf16 storage with f64 compute
    assert hdiff(lib, F32, F32X2)[0] == UNSUPPORTED  # pairs need f64 storage
    assert hdiff(lib, F32, FIX64)[0] == UNSUPPORTED
    assert hdiff(lib, F64, F64, nk=0) == (OK, 0.0)  # empty domain: no launch, time 0


def test_vadv_argument_checks(lib):
    assert vadv(lib, F64, F64, stage=NULL) == INVALID
    assert vadv(lib, F64, F64, shift=(1, 1)) == INVALID and "shift" in _msg()
    assert vadv(lib, F64, F64, shift=(2, 0)) == INVALID
    assert vadv(lib, F64, F64, nk=1) == INVALID and "2 levels" in _msg()
    assert vadv(lib, BF16, F64) == UNSUPPORTED
    assert vadv(lib, F64, FIX64) == UNSUPPORTED  # fixed point is hdiff only


def test_vadv3_checks(lib):
    arr = ctypes.c_void_p * 3
    good = arr(P, P, P)
    holey = arr(P, NULL, P)

    def call(stage=good, out=good, storage=F64, compute=F64, nk=4):
        return lib.sb_vadv3(storage, compute, stage, good, good, good, P, out, None, None, 8, 8, nk, 1, 10, 100,
                            None, None, None)

    assert call(stage=holey) == INVALID and "component 1" in _msg()
    assert call(out=holey) == INVALID
    assert lib.sb_vadv3(F64, F64, None, good, good, good, P, good, None, None, 8, 8, 4, 1, 10, 100,
                        None, None, None) == INVALID
    assert call(nk=1) == INVALID and "2 levels" in _msg()
    assert call(storage=BF16, compute=F64) == UNSUPPORTED
    assert call(nk=0) == OK  # empty domain: no launch


def test_copy_helpers_checks(lib):
    assert lib.sb_memcpy_sm(NULL, P, 16, None) == INVALID
    assert lib.sb_memcpy_sm(NULL, NULL, 0, None) == OK
    assert lib.sb_debug_soft_f64(4, P, P, P, 8, None) == INVALID and "reciprocal" in _msg()
    assert lib.sb_debug_soft_f64(0, P, NULL, P, 8, None) == INVALID  # add needs b
    assert lib.sb_debug_soft_f64(3, P, NULL, P, 0, None) == OK  # the reciprocal ignores b


def test_basic_and_stream_checks(lib):
    assert lib.sb_laplacian(F64, F64, P, P, 8, 8, 4, 1, 10, 100, 9, None, None, None) == INVALID
    assert lib.sb_average(F64, F64, P, P, 8, 8, 4, 1, 10, 100, 3, 0, None, None, None) == INVALID
    assert lib.sb_copy(F64, NULL, P, 8, 8, 4, 1, 10, 100, None, None, None) == INVALID
    assert lib.sb_empty(-1, 1, 1, None, None, None) == INVALID
    t = ctypes.c_double(-1.0)
    assert lib.sb_empty(0, 5, 5, None, None, ctypes.byref(t)) == OK and t.value == 0.0
    assert lib.sb_stream_op(9, F64, P, P, P, 3.0, 16, None, None, None) == INVALID
    assert lib.sb_stream_op(_native.STREAM_TRIAD, BF16, P, P, P, 3.0, 16, None, None, None) == UNSUPPORTED
    assert lib.sb_stream_op(_native.STREAM_COPY, F64, P, NULL, P, 3.0, 0, None, None, None) == OK


def test_batch_and_fill_checks(lib):
    h = ctypes.c_void_p()
    assert lib.sb_batch_create(ctypes.byref(h), F64, F64, 0, 80, None) == INVALID
    assert lib.sb_batch_create(ctypes.byref(h), F64, F64, 4, 1, None) == INVALID  # max_nk >= 2
    assert lib.sb_batch_create(ctypes.byref(h), BF16, F64, 4, 80, None) == UNSUPPORTED
    from stencil_benchmarks_gb300.serving import SbFillDesc

    bad = (SbFillDesc * 1)(SbFillDesc(0x1000, -5, 1, 0.0, 1.0, F64, 0))
    assert lib.sb_fill_batch(ctypes.cast(bad, ctypes.c_void_p), 1, P, None) == INVALID
    bad[0] = SbFillDesc(0x1000, 5, 1, 0.0, 1.0, 7, 0)
    assert lib.sb_fill_batch(ctypes.cast(bad, ctypes.c_void_p), 1, P, None) == INVALID
    assert lib.sb_fill_batch(None, 0, None, None) == OK  # nothing to fill


def test_error_text_is_per_call(lib):
    assert hdiff(lib, F64, F64, inp=NULL)[0] == INVALID
    assert _msg()
    assert hdiff(lib, F64, F64, nk=0)[0] == OK
    assert _msg() == ""  # a successful call clears the previous message
