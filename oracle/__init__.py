"""CPU oracle for the GB300 stencil backend -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, the arithmetic that the reference
(GridTools/stencil_benchmarks 0.11.0) uses to verify its stencils:

* ``oracle.stencils``  -- numpy restatement of ``Stencil.verify_stencil`` for
  copy, averages, Laplacian, horizontal diffusion and vertical advection, plus
  the STREAM kernels and bf16 rounding helpers.
* ``oracle.cport``     -- ctypes binding of ``oracle/csrc/oracle.c``, a plain C
  (OpenMP) restatement of hdiff / vadv used as the timed CPU baseline.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline
and reference arms) may import this package, and only to check results or as
the timed CPU baseline.  The product package ``stencil_benchmarks_gb300`` never
imports it; it has no CPU compute path at all.

Parity pin: every function here is checked bit-for-bit against golden vectors
captured from the reference's own ``verify_stencil`` / numpy backend
(``tests/golden/make_golden.py``, ``tests/test_oracle_golden.py``).
"""
