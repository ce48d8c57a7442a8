"""Benchmarks of the GB300 backend, laid out like the reference's collection so
that command paths match (``stencils gb300 horizontal-diffusion j-scan``,
``stream gb300 native``)."""

from . import stencils, stream

__all__ = ["stencils", "stream"]
