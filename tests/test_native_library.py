"""The C ABI library builds, loads without a GPU and exports every entry
point that ``include/sbgb300.h`` declares (no compute calls here)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from stencil_benchmarks_gb300 import _native
from stencil_benchmarks_gb300 import build as sbbuild

HEADER = Path(__file__).resolve().parent.parent / "include" / "sbgb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    path = sbbuild.build()
    assert path.exists()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("sb_hdiff", "sb_vadv", "sb_copy", "sb_laplacian", "sb_average", "sb_stream_op",
                     "sb_last_error", "sb_malloc", "sb_free"):
        assert required in names


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared_functions() if not hasattr(library, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_device_count_without_gpu_is_not_an_error(library):
    # loading and querying must work on a machine without a GPU; on a GPU
    # machine this just reports the devices.
    _native.lib()
    assert _native.device_count() >= 0


def test_invalid_arguments_are_rejected_before_any_launch(library):
    """Argument validation runs on the host and never touches a device."""
    lib = _native.lib()
    rc = lib.sb_hdiff(0, 0, None, None, None, -1, 1, 1, 1, 1, 1, None, None, None)
    assert rc == _native.SB_ERR_INVALID
    assert "negative domain" in _native.last_error()
    rc = lib.sb_vadv(0, 0, None, None, None, None, None, None, None, None, 4, 4, 4, 1, 4, 16, 2, 0,
                     None, None, None)
    assert rc == _native.SB_ERR_INVALID
    rc = lib.sb_stream_op(4, 2, None, None, None, 3.0, 10, None, None, None)
    assert rc == _native.SB_ERR_UNSUPPORTED
    rc = lib.sb_laplacian(0, 0, None, None, 4, 4, 4, 1, 4, 16, 9, None, None, None)
    assert rc == _native.SB_ERR_INVALID


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setenv("SBGB300_LIBRARY", str(tmp_path / "nope.so"))
    with pytest.raises(_native.NativeLibraryError):
        _native.lib()
    monkeypatch.setattr(_native, "_lib", None)
