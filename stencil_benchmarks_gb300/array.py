"""Padded, aligned, layout-permuted host arrays.

Same layout rules as the reference's ``tools/array.py:alloc_array``
(stencil_benchmarks/tools/array.py:53-177), so fields have identical strides
and alignment whichever backend allocates them:

* ``layout[d]`` ranks dimension ``d``: ``ndim-1`` is the unit-stride axis,
  ``0`` the outermost;
* with a non-zero ``alignment`` (bytes) the unit-stride extent is padded so
  that every larger stride is a multiple of ``alignment``, and the element
  at ``index_to_align`` (the first interior point for stencil fields) starts
  on an ``alignment`` boundary.

Element types are "float64", "float32" and "bfloat16"; bfloat16 fields are
held on the host as their 16-bit patterns (numpy ``uint16``), because numpy
has no bfloat16 type.
"""

from __future__ import annotations

import ctypes
from typing import Callable, Optional, Sequence

import numpy as np

_STORAGE = {
    "float64": np.dtype(np.float64),
    "float32": np.dtype(np.float32),
    "bfloat16": np.dtype(np.uint16),
}

_cache_offset_counter = 0


def storage_numpy_dtype(storage: str) -> np.dtype:
    try:
        return _STORAGE[storage]
    except KeyError:
        raise ValueError(f"unsupported storage type {storage!r}") from None


def element_size(storage: str) -> int:
    return storage_numpy_dtype(storage).itemsize


def layout_strides(shape: Sequence[int], itemsize: int, layout: Sequence[int], alignment: int = 0):
    """Byte strides and total bytes for ``shape`` under ``layout``/``alignment``."""
    ndim = len(shape)
    if sorted(layout) != list(range(ndim)):
        raise ValueError("invalid layout specification")
    if alignment < 0:
        raise ValueError("alignment must be non-negative")
    strides = [0] * ndim
    running = itemsize
    for rank in reversed(range(ndim)):
        dim = list(layout).index(rank)
        strides[dim] = running
        running *= shape[dim]
        if rank == ndim - 1 and alignment:
            running = -(-running // alignment) * alignment
    return tuple(strides), running


def alloc_array(
    shape: Sequence[int],
    dtype,
    layout: Sequence[int],
    alignment: int = 0,
    index_to_align: Optional[Sequence[int]] = None,
    alloc: Optional[Callable[[int], object]] = None,
    apply_offset: bool = False,
    cache_sets: int = 64,
    cache_line: int = 64,
) -> np.ndarray:
    """Allocate an uninitialised numpy array with the reference's layout rules.

    ``alloc(nbytes)`` must return a writable buffer object (default:
    ``bytearray``).  ``apply_offset`` shifts successive allocations by
    multiples of the cache line (or alignment) to spread them over cache sets.
    """
    global _cache_offset_counter
    shape = tuple(int(s) for s in shape)
    dtype = storage_numpy_dtype(dtype) if isinstance(dtype, str) and dtype in _STORAGE else np.dtype(dtype)
    index_to_align = (0,) * len(shape) if index_to_align is None else tuple(index_to_align)
    if not len(shape) == len(layout) == len(index_to_align):
        raise ValueError("dimension mismatch")
    strides, total = layout_strides(shape, dtype.itemsize, layout, int(alignment))
    offset = 0
    if apply_offset:
        step = max(cache_line, alignment)
        offset = (_cache_offset_counter % cache_sets) * (1 << (step.bit_length() - 1))
        _cache_offset_counter += 1
    alloc = alloc or bytearray
    buffer = alloc(total + int(alignment) + offset)
    if alignment:
        base = ctypes.addressof(ctypes.c_char.from_buffer(buffer))
        target = base + sum(s * i for s, i in zip(strides, index_to_align)) + offset
        offset += (-target) % alignment
    return np.ndarray(shape=shape, dtype=dtype, buffer=buffer, offset=offset, strides=strides)


def nbytes(data: np.ndarray) -> int:
    """Bytes a linear copy of ``data`` must move, padding included."""
    last = int(np.sum((np.array(data.shape) - 1) * np.array(data.strides)))
    return last + data.itemsize
