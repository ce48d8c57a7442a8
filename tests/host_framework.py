"""Access to the reference's ``stencil_benchmarks`` package (the host
framework the GB300 benchmark classes plug into) for the tests.

``require()`` loads it through ``stencil_benchmarks_gb300.host`` and skips
the calling test with the reason when no copy is available (a checkout where
``__graft_entry__.build()`` has not installed ``baseline/_ref``)."""

from __future__ import annotations

import pytest


def require():
    from stencil_benchmarks_gb300 import host

    try:
        return host.load()
    except host.HostFrameworkMissing as err:
        pytest.skip(str(err))
