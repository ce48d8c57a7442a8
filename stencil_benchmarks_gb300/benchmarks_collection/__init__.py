"""Benchmarks of the GB300 backend, laid out like the reference's collection so
that the reference's CLI derives the command paths ``stencils gb300
horizontal-diffusion tma-tile``, ``stream gb300 native``, ... from the module
names (stencil_benchmarks/cli.py:47-50).

Importing this package loads the reference's ``stencil_benchmarks`` package
(``stencil_benchmarks_gb300.host``): every class here derives from its
``Benchmark`` / ``Stencil`` classes and registers in its ``REGISTRY``."""

from ..host import load as _load_host_framework

_load_host_framework()

from . import stencils, stream  # noqa: E402

__all__ = ["stencils", "stream"]
