"""Every registered benchmark, run through the Benchmark API with verification
(the reference's test_benchmarks_collection.py strategy, here on the GPU and
with the CPU oracle installed as the verifier)."""

from __future__ import annotations

import pytest

from stencil_benchmarks_gb300 import benchmark
from stencil_benchmarks_gb300 import benchmarks_collection  # noqa: F401
from stencil_benchmarks_gb300.benchmarks_collection.stencils.gb300 import (
    basic,
    horizontal_diffusion,
    vertical_advection,
)
from stencil_benchmarks_gb300.benchmarks_collection.stream import gb300 as stream

pytestmark = pytest.mark.gpu

OURS = sorted((b for b in benchmark.REGISTRY if b.__module__.startswith("stencil_benchmarks_gb300.")),
              key=lambda b: (b.__module__, b.__name__))


@pytest.mark.parametrize("bmark", OURS, ids=lambda b: f"{b.__module__.split('.')[-1]}.{b.__name__}")
def test_default_construction_runs_and_verifies(bmark, lib):
    instance = bmark()
    results = instance.run()
    results = results if isinstance(results, list) else [results]
    assert all(r["time"] > 0 for r in results)
    # a second execution (the data set cycles / STREAM reruns)
    instance.run()


@pytest.mark.parametrize("cls", [horizontal_diffusion.JScan, horizontal_diffusion.Tile, horizontal_diffusion.TmaTile,
                                 horizontal_diffusion.VectorScan])
@pytest.mark.parametrize("dtype", ["float64", "float32", "bfloat16"])
def test_hdiff_benchmark_forms(cls, dtype, lib):
    b = cls(domain=(100, 77, 9), halo=(2, 2, 0), dtype=dtype, data_sets=2, alignment=0)
    for _ in range(3):
        r = b.run()
        assert r["gpoints_per_s"] > 0 and r["bandwidth"] > 0


@pytest.mark.parametrize("cls", [vertical_advection.SharedMem, vertical_advection.GlobalScratch,
                                 vertical_advection.Slab, vertical_advection.NoAlloc])
@pytest.mark.parametrize("all_components", [False, True])
def test_vadv_benchmark_forms(cls, all_components, lib):
    b = cls(domain=(64, 40, 30), halo=(1, 1, 1), all_components=all_components)
    b.run()


@pytest.mark.parametrize("dtype", ["float32", "bfloat16"])
@pytest.mark.parametrize("all_components", [False, True])
def test_vadv_tensor_mem_benchmark(dtype, all_components, lib):
    """The reference's numpy verification of float32 / bfloat16-storage runs
    with the factors in tensor memory."""
    b = vertical_advection.TensorMem(domain=(64, 40, 30), halo=(1, 1, 1), dtype=dtype,
                                     all_components=all_components)
    for _ in range(2):
        b.run()
    with pytest.raises(benchmark.ParameterError):
        vertical_advection.TensorMem(domain=(64, 40, 30), halo=(1, 1, 1), dtype="float64")


@pytest.mark.parametrize("cls,compute", [(horizontal_diffusion.JScan, "fixed64"),
                                         (horizontal_diffusion.JScan, "float32x2"),
                                         (horizontal_diffusion.Tile, "float32x2"),
                                         (vertical_advection.SharedMem, "float32x2"),
                                         (vertical_advection.Slab, "float32x2")])
def test_fast_float64_forms_verify(cls, compute, lib):
    """The fast float64 forms pass the reference's own float64 tolerance."""
    halo = (2, 2, 0) if cls.__module__.endswith("horizontal_diffusion") else (1, 1, 0)
    cls(domain=(90, 70, 12), halo=halo, compute_dtype=compute, data_sets=2).run()


def test_fast_forms_parameter_checks(lib):
    with pytest.raises(benchmark.ParameterError):
        vertical_advection.SharedMem(domain=(16, 16, 8), halo=(1, 1, 0), compute_dtype="fixed64")
    with pytest.raises(benchmark.ParameterError):
        horizontal_diffusion.JScan(domain=(16, 16, 8), halo=(2, 2, 0), dtype="float32", compute_dtype="float32x2")


def test_vadv_fp32_storage_with_fp64_solve(lib):
    vertical_advection.SharedMem(domain=(64, 40, 30), halo=(1, 1, 0), dtype="float32",
                                 compute_dtype="float64").run()


@pytest.mark.parametrize("cls,kw", [
    (basic.Empty, {"halo": (1, 1, 1)}),
    (basic.Laplacian, {"along_z": True, "halo": (1, 1, 1)}),
    (basic.OnesidedAverage, {"axis": 2, "halo": (1, 1, 1)}),
    (basic.SymmetricAverage, {"axis": 1, "halo": (1, 1, 1)}),
    (basic.Copy, {"layout": (0, 1, 2), "alignment": 64}),
])
def test_basic_benchmark_variants(cls, kw, lib):
    cls(domain=(50, 30, 20), **kw).run()


def test_wall_timers_and_dry_runs(lib):
    b = horizontal_diffusion.JScan(domain=(64, 64, 8), halo=(2, 2, 0), timers="wall", dry_runs=2)
    assert b.run()["time"] > 0


def test_stream_native(lib):
    res = stream.Native(array_size=1 << 20, ntimes=4, dtype="float32").run()
    assert [r["name"] for r in res] == ["copy", "scale", "add", "triad"]
    assert all(r["bandwidth"] > 0 and r["time"] <= r["avg-time"] <= r["max-time"] for r in res)


def test_cli_runs_a_benchmark(lib, tmp_path):
    pytest.importorskip("click")
    from stencil_benchmarks_gb300 import cli

    out = tmp_path / "res.csv"
    cli.main(args=["-e", "2", "-o", str(out), "stencils", "gb300", "horizontal-diffusion", "j-scan",
                   "--domain", "[32,64]", "32", "8", "--halo", "2", "2", "0"], standalone_mode=False)
    lines = out.read_text().splitlines()
    assert len(lines) == 1 + 4  # header + 2 domains x 2 executions


@pytest.mark.parametrize("cls,kw", [
    (horizontal_diffusion.JScan, {"halo": (2, 2, 0)}),
    (horizontal_diffusion.TmaTile, {"halo": (2, 2, 0)}),
    (horizontal_diffusion.VectorScan, {"halo": (2, 2, 0), "dtype": "bfloat16"}),
    (vertical_advection.SharedMem, {"halo": (1, 1, 0)}),
    (vertical_advection.Slab, {"halo": (1, 1, 0)}),
    (vertical_advection.TensorMem, {"halo": (1, 1, 0)}),
])
def test_autotune_parameter(cls, kw, lib):
    """autotune=True times the implementation's candidate shapes during setup,
    runs the fastest (reported as `tune`) and still verifies."""
    b = cls(domain=(96, 64, 40), autotune=True, **kw)
    for _ in range(2):
        r = b.run()
        assert r["time"] > 0 and isinstance(r["tune"], str) and r["tune"]
