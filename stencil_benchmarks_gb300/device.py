"""Device memory, streams and 3D fields on the GPU.

``DeviceBuffer`` owns one ``cudaMalloc`` allocation made by the native
library (freed by a finalizer, like the reference's ``api.Runtime.malloc``,
stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/api.py:54-78).
``Field`` describes a halo'd 3D array inside a buffer: its shape, element
strides and element type, and gives the address of the first interior point
that the C ABI expects (reference: compilation.data_ptr, tools/compilation.py:273-282).
"""

from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass

import numpy as np

from . import _native
from .array import element_size, storage_numpy_dtype


class DeviceBuffer:
    """A device allocation of ``nbytes`` bytes, freed when garbage collected."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        ptr = ctypes.c_void_p()
        _native.call("sb_malloc", ctypes.byref(ptr), ctypes.c_size_t(self.nbytes))
        self.ptr = ptr.value or 0
        self._finalizer = weakref.finalize(self, DeviceBuffer._release, self.ptr)

    @staticmethod
    def _release(ptr):
        if ptr:
            try:
                _native.lib().sb_free(ctypes.c_void_p(ptr))
            except Exception:  # noqa: BLE001 - interpreter shutdown
                pass

    def free(self):
        self._finalizer()
        self.ptr = 0

    def __int__(self):
        return self.ptr


class PinnedBuffer:
    """Page-locked host memory (for asynchronous copies), exposed as numpy."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        ptr = ctypes.c_void_p()
        _native.call("sb_malloc_host", ctypes.byref(ptr), ctypes.c_size_t(max(self.nbytes, 1)))
        self.ptr = ptr.value or 0
        self._finalizer = weakref.finalize(self, PinnedBuffer._release, self.ptr)

    @staticmethod
    def _release(ptr):
        if ptr:
            try:
                _native.lib().sb_free_host(ctypes.c_void_p(ptr))
            except Exception:  # noqa: BLE001
                pass

    def array(self, dtype, shape, strides=None, offset=0):
        raw = (ctypes.c_byte * max(self.nbytes, 1)).from_address(self.ptr)
        return np.ndarray(shape, dtype=dtype, buffer=raw, offset=offset, strides=strides)


class Stream:
    """A non-blocking CUDA stream owned by the native library."""

    def __init__(self):
        ptr = ctypes.c_void_p()
        _native.call("sb_stream_create", ctypes.byref(ptr))
        self.handle = ptr.value
        self._finalizer = weakref.finalize(self, Stream._release, self.handle)

    @staticmethod
    def _release(handle):
        if handle:
            try:
                _native.lib().sb_stream_destroy(ctypes.c_void_p(handle))
            except Exception:  # noqa: BLE001
                pass

    def synchronize(self):
        _native.call("sb_stream_synchronize", ctypes.c_void_p(self.handle))

    @property
    def as_parameter(self):
        return ctypes.c_void_p(self.handle)


class Event:
    def __init__(self):
        ptr = ctypes.c_void_p()
        _native.call("sb_event_create", ctypes.byref(ptr))
        self.handle = ptr.value
        self._finalizer = weakref.finalize(self, Event._release, self.handle)

    @staticmethod
    def _release(handle):
        if handle:
            try:
                _native.lib().sb_event_destroy(ctypes.c_void_p(handle))
            except Exception:  # noqa: BLE001
                pass

    def record(self, stream=None):
        _native.call("sb_event_record", ctypes.c_void_p(self.handle), _stream_arg(stream))

    def synchronize(self):
        _native.call("sb_event_synchronize", ctypes.c_void_p(self.handle))

    def elapsed(self, end: "Event") -> float:
        out = ctypes.c_double()
        _native.call("sb_event_elapsed", ctypes.c_void_p(self.handle), ctypes.c_void_p(end.handle),
                     ctypes.byref(out))
        return out.value


def _stream_arg(stream):
    if stream is None:
        return None
    if isinstance(stream, Stream):
        return stream.as_parameter
    return ctypes.c_void_p(int(stream))


def copy_to_device(dst_ptr: int, host: np.ndarray, nbytes: int | None = None, stream=None):
    nbytes = host.nbytes if nbytes is None else nbytes
    if stream is None:
        _native.call("sb_memcpy", ctypes.c_void_p(dst_ptr), ctypes.c_void_p(host.ctypes.data),
                     ctypes.c_size_t(nbytes), _native.H2D)
    else:
        _native.call("sb_memcpy_async", ctypes.c_void_p(dst_ptr), ctypes.c_void_p(host.ctypes.data),
                     ctypes.c_size_t(nbytes), _native.H2D, _stream_arg(stream))


def copy_to_host(host: np.ndarray, src_ptr: int, nbytes: int | None = None, stream=None):
    nbytes = host.nbytes if nbytes is None else nbytes
    if stream is None:
        _native.call("sb_memcpy", ctypes.c_void_p(host.ctypes.data), ctypes.c_void_p(src_ptr),
                     ctypes.c_size_t(nbytes), _native.D2H)
    else:
        _native.call("sb_memcpy_async", ctypes.c_void_p(host.ctypes.data), ctypes.c_void_p(src_ptr),
                     ctypes.c_size_t(nbytes), _native.D2H, _stream_arg(stream))


def l2_flush(stream=None):
    _native.call("sb_l2_flush", _stream_arg(stream))


@dataclass
class Field:
    """A halo'd 3D array in device memory.

    ``strides`` are in elements; ``offset`` is the byte offset of element
    (0, 0, 0) inside ``buffer``.  ``storage`` is "float64", "float32" or
    "bfloat16".
    """

    buffer: DeviceBuffer
    shape: tuple
    strides: tuple
    storage: str
    halo: tuple
    offset: int = 0

    @property
    def itemsize(self) -> int:
        return element_size(self.storage)

    @property
    def base_ptr(self) -> int:
        return self.buffer.ptr + self.offset

    @property
    def interior_ptr(self) -> int:
        """Address of the first interior point (the C ABI's field pointer)."""
        off = sum(s * h for s, h in zip(self.strides, self.halo)) * self.itemsize
        return self.base_ptr + off

    @property
    def span_bytes(self) -> int:
        """Bytes from element (0,0,0) to one past the last element."""
        last = sum((n - 1) * s for n, s in zip(self.shape, self.strides))
        return (last + 1) * self.itemsize

    @classmethod
    def like_host(cls, host: np.ndarray, storage: str, halo) -> "Field":
        """Allocate a device field with the same shape/strides as ``host``."""
        itemsize = element_size(storage)
        strides = tuple(s // itemsize for s in host.strides)
        last = sum((n - 1) * s for n, s in zip(host.shape, strides))
        nbytes = (last + 1) * itemsize if host.size else 0
        buf = DeviceBuffer(max(nbytes, 1))
        return cls(buf, tuple(host.shape), strides, storage, tuple(halo))

    def upload(self, host: np.ndarray, stream=None):
        """Copy the whole span of ``host`` (padding included) to the device."""
        assert tuple(s // self.itemsize for s in host.strides) == self.strides
        if host.size:
            copy_to_device(self.base_ptr, _span_view(host), self.span_bytes, stream)

    def download(self, host: np.ndarray, stream=None):
        assert tuple(s // self.itemsize for s in host.strides) == self.strides
        if host.size:
            copy_to_host(_span_view(host), self.base_ptr, self.span_bytes, stream)


def _span_view(host: np.ndarray) -> np.ndarray:
    """A 1D byte view starting at host[0,0,0] covering the array's span."""
    assert all(s > 0 for s in host.strides), "negative strides are not supported"
    last = sum((n - 1) * s for n, s in zip(host.shape, host.strides))
    nbytes = last + host.itemsize
    raw = (ctypes.c_byte * nbytes).from_address(host.ctypes.data)
    return np.frombuffer(raw, dtype=np.uint8)


def host_storage_dtype(storage: str):
    return storage_numpy_dtype(storage)
