"""Shared pytest configuration.

Markers:
  gpu  -- needs a CUDA device and the built native library; run with
          ``pytest -m gpu``.  Everything else runs on a CPU-only machine.
"""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libsbgb300.so")


def golden_cases():
    return json.loads((GOLDEN / "cases.json").read_text())


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz") as data:
        return {k: data[k] for k in data.files}


@pytest.fixture(scope="session")
def golden():
    return golden_cases()


def gpu_available() -> bool:
    if os.environ.get("SB_FORCE_NO_GPU"):
        return False
    try:
        from stencil_benchmarks_gb300 import _native

        return _native.device_count() > 0
    except Exception:  # noqa: BLE001 - any failure means "no usable GPU"
        return False


@pytest.fixture(scope="session")
def lib():
    """The loaded native library; GPU tests fail (not skip) if it is missing."""
    from stencil_benchmarks_gb300 import _native

    return _native.lib()
