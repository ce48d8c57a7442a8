"""The Benchmark/Parameter contract (same behaviour as the reference's
stencil_benchmarks/benchmark.py, checked the way its test_benchmark.py does)."""

from __future__ import annotations

import numpy as np
import pytest

from stencil_benchmarks_gb300 import array as sbarray
from stencil_benchmarks_gb300 import benchmark


class SomeBenchmark(benchmark.Benchmark):
    parameter1 = benchmark.Parameter("some parameter", False)
    parameter2 = benchmark.Parameter("some other parameter", 1)

    def setup(self):
        self.somevalue = self.parameter2 // 2

    def run(self):
        return self.somevalue


class DerivedBenchmark(SomeBenchmark):
    parameter3 = benchmark.Parameter("third parameter", "0")

    def setup(self):
        super().setup()
        self.paramsum = sum(int(p) for p in self.parameters.values())

    def run(self):
        return self.paramsum


def test_registration():
    assert SomeBenchmark in benchmark.REGISTRY
    assert DerivedBenchmark in benchmark.REGISTRY


def test_params_and_inheritance():
    assert SomeBenchmark.parameters == {
        "parameter1": benchmark.Parameter("some parameter", False),
        "parameter2": benchmark.Parameter("some other parameter", 1),
    }
    assert DerivedBenchmark.parameters == {
        "parameter1": benchmark.Parameter("some parameter", False, bool),
        "parameter2": benchmark.Parameter("some other parameter", 1, int),
        "parameter3": benchmark.Parameter("third parameter", "0", str),
    }


def test_init_validates_and_calls_setup():
    b = SomeBenchmark(parameter1=True, parameter2=42)
    assert (b.parameter1, b.parameter2, b.somevalue) == (True, 42, 21)
    assert b.parameters == {"parameter1": True, "parameter2": 42}
    with pytest.raises(benchmark.ParameterError):
        SomeBenchmark(parameter1=3, parameter2="42")
    with pytest.raises(ValueError):
        SomeBenchmark(nonexistent=1)


def test_derived_init_run_and_reassign():
    b = DerivedBenchmark(parameter1=True, parameter2=42, parameter3="5")
    assert b.paramsum == 48 and b.run() == 48 and b() == 48
    b.parameter1 = False
    assert b.parameter1 is False and b.parameters["parameter1"] is False
    with pytest.raises(benchmark.ParameterError):
        b.parameter1 = 3


def test_parameter_rules():
    with pytest.raises(ValueError):
        benchmark.Parameter("no default, no type")
    with pytest.raises(ValueError):
        benchmark.Parameter("mixed", (1, 2.0))
    p = benchmark.Parameter("tuple", (1, 2, 3))
    assert p.validate((4, 5, 6)) == (4, 5, 6)
    for bad in ((1, 2), (1, 2, 3.0), 7):
        with pytest.raises(benchmark.ParameterError):
            p.validate(bad)
    c = benchmark.Parameter("choice", "a", choices=["a", "b"])
    with pytest.raises(benchmark.ParameterError):
        c.validate("c")
    r = benchmark.Parameter("required", dtype=str, nargs=1)
    with pytest.raises(benchmark.ParameterError):
        r.validate(None)


def test_defining_parameters_attribute_is_rejected():
    with pytest.raises(AttributeError):

        class Bad(benchmark.Benchmark):  # noqa: F841
            parameters = {}

            def run(self):
                return 0


# -- layout rules of tools/array.py (its doctests, restated) -------------------


def test_alloc_array_layouts_and_alignment():
    x = sbarray.alloc_array((2, 3), "int32", (1, 0))
    assert x.strides == (4, 8)
    x = sbarray.alloc_array((2, 3), "int32", (0, 1))
    assert x.strides == (12, 4)
    x = sbarray.alloc_array((2, 3), "int32", (0, 1), alignment=64)
    assert x.strides == (64, 4) and x.ctypes.data % 64 == 0
    assert sbarray.nbytes(x) == 76
    # the first interior point is the aligned one
    f = sbarray.alloc_array((20, 10, 5), "float64", (2, 1, 0), alignment=128, index_to_align=(3, 3, 1))
    assert (f.ctypes.data + f.strides[0] * 3 + f.strides[1] * 3 + f.strides[2]) % 128 == 0
    assert f.strides[1] % 128 == 0 and f.strides[2] % 128 == 0
    assert sbarray.alloc_array((4, 4, 4), "bfloat16", (2, 1, 0)).dtype == np.uint16


def test_stencil_benchmarks_need_a_gpu_or_fail_validation_cleanly():
    """On a machine without a GPU every registered stencil benchmark refuses
    construction with ParameterError (the CLI skips those with -s), like the
    reference's cuda_hip benchmarks without --gpu-architecture."""
    import os

    from stencil_benchmarks_gb300 import _native
    from stencil_benchmarks_gb300 import benchmarks_collection  # noqa: F401

    if _native.device_count() > 0 and not os.environ.get("SB_FORCE_NO_GPU"):
        pytest.skip("a GPU is present")
    ours = [b for b in benchmark.REGISTRY if b.__module__.startswith("stencil_benchmarks_gb300.")]
    assert len(ours) >= 10
    for bmark in ours:
        with pytest.raises(benchmark.ParameterError):
            bmark(verify=False) if "verify" in bmark.parameters else bmark()
