"""Where a stencil's ``verify=True`` gets its CPU check from.

The reference verifies every run by recomputing the stencil in numpy inside
its ``Stencil`` base classes (stencil_benchmarks/benchmarks_collection/
stencils/base.py:151-166, 180-501).  This package computes only on the GPU and
ships no CPU implementation, so verification is supplied from outside and
registered here per stencil kind:

* with the reference installed, ``reference_bridge.install()`` registers the
  reference's own ``verify_stencil`` methods;
* the test suite registers its CPU oracle.

A verifier is ``fn(stencil, data_before, data_after)`` and raises
``validation.ValidationError`` on a mismatch.  Kinds: "copy",
"onesided_average", "symmetric_average", "laplacian",
"horizontal_diffusion", "vertical_advection", and "empty", which is
registered here: the reference's EmptyStencil checks nothing
(stencils/base.py:175-177).
"""

from __future__ import annotations

from typing import Callable, Dict, Optional

_VERIFIERS: Dict[str, Callable] = {}


def register(kind: str, fn: Callable) -> None:
    _VERIFIERS[kind] = fn


def unregister(kind: str) -> None:
    _VERIFIERS.pop(kind, None)


def _nothing_to_check(stencil, data_before, data_after):
    pass


_VERIFIERS["empty"] = _nothing_to_check


def get(kind: str) -> Optional[Callable]:
    return _VERIFIERS.get(kind)


def registered() -> Dict[str, Callable]:
    return dict(_VERIFIERS)
