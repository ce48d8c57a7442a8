"""The precision report's forms on a small random domain (the full
512 x 512 x 80 report is ``python -m tests.precision_report``).

The float64-storage forms are checked against the float64 oracle:
  float64 / float64    bit-identical (error 0)
  float64 / fixed64    <= 2^-50 of the field scale (hdiff)
  float64 / float32x2  <= 1e-12 (hdiff) / 1e-10 (vadv) of the field scale
The quantised-storage forms are checked on their arithmetic alone, against
the oracle in their compute type on their own stored inputs:
  float32 / float32    bit-identical
  float32 / float64    <= 2^-24 of the scale (the final rounding to float32)
  bfloat16 / float32   <= 2^-8 of the scale (the final rounding to bfloat16)
Their total error against the float64 oracle on the float64 draws is
reported, not bounded: hdiff's limiter flips, and the random vadv systems
include nearly singular columns (the diagonal 0.15 - acol - ccol can
approach 0) that amplify the rounding of the stored inputs themselves.
"""

from __future__ import annotations

import pytest

from tests import precision_report as pr

pytestmark = pytest.mark.gpu

F64 = {("float64", "float64"): 0.0, ("float64", "fixed64"): 2.0**-50}
PAIR = {"hdiff": 1e-12, "vadv": 1e-10}
ARITH = {("float32", "float32"): 0.0, ("float32", "float64"): 2.0**-24, ("bfloat16", "float32"): 2.0**-8}


@pytest.mark.parametrize("which", ["hdiff", "vadv"])
def test_precision_bounds(which, lib):
    domain = (70, 45, 24)
    rep = pr.hdiff_report(domain, reps=1) if which == "hdiff" else pr.vadv_report(domain, reps=1)
    for row in rep["forms"]:
        form = (row["storage"], row["compute"])
        assert row["gpoints_s"] > 0 and row["bytes_moved"] > 0
        if form[0] == "float64":
            bound = PAIR[which] if form[1] == "float32x2" else F64[form]
            assert row["err_max_scale"] <= bound, (which, form, row)
        else:
            arith = row["vs_oracle_on_quantised_inputs"]["err_max_scale"]
            assert arith <= ARITH[form], (which, form, arith)
    if which == "hdiff":
        assert 0 <= rep["limiter_ties_exact_zero"] <= rep["limiter_decisions"]
