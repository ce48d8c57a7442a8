"""The GB300 backend inside the reference's own Benchmark API and CLI (CPU).

The benchmark classes derive from the reference's ``Benchmark`` and
``Stencil`` classes, so they must appear in its ``REGISTRY``
(stencil_benchmarks/benchmark.py:140-164) under the command paths its CLI
derives (stencil_benchmarks/cli.py:47-50), with the reference's parameters
plus this backend's additions, and refuse construction cleanly without a GPU.
"""

from __future__ import annotations

import ctypes
import mmap

import numpy as np
import pytest

from stencil_benchmarks_gb300 import array as sbarray
from tests.host_framework import require


@pytest.fixture(scope="module")
def ref():
    require()
    import stencil_benchmarks.benchmarks_collection  # noqa: F401
    from stencil_benchmarks import benchmark, cli

    from stencil_benchmarks_gb300 import benchmarks_collection  # noqa: F401

    return benchmark, cli


def _ours(benchmark):
    return sorted((b for b in benchmark.REGISTRY if b.__module__.startswith("stencil_benchmarks_gb300.")),
                  key=lambda b: (b.__module__, b.__name__))


def test_gb300_classes_are_in_the_reference_registry(ref):
    benchmark, cli = ref
    paths = {" ".join(cli._cli_command(b)) for b in _ours(benchmark)}
    assert paths == {
        "stencils gb300 basic copy", "stencils gb300 basic empty", "stencils gb300 basic laplacian",
        "stencils gb300 basic onesided-average", "stencils gb300 basic symmetric-average",
        "stencils gb300 horizontal_diffusion j-scan", "stencils gb300 horizontal_diffusion tile",
        "stencils gb300 horizontal_diffusion tma-tile", "stencils gb300 horizontal_diffusion vector-scan",
        "stencils gb300 vertical_advection global-scratch", "stencils gb300 vertical_advection no-alloc",
        "stencils gb300 vertical_advection shared-mem", "stencils gb300 vertical_advection slab",
        "stencils gb300 vertical_advection tensor-mem", "stream gb300 native",
    }


def test_classes_derive_from_the_reference_stencils(ref):
    from stencil_benchmarks.benchmarks_collection.stencils import base

    from stencil_benchmarks_gb300.benchmarks_collection.stencils.gb300 import (
        basic,
        horizontal_diffusion,
        vertical_advection,
    )

    for cls in (horizontal_diffusion.TmaTile, horizontal_diffusion.JScan, horizontal_diffusion.Tile,
                horizontal_diffusion.VectorScan):
        assert issubclass(cls, base.HorizontalDiffusionStencil)
        assert cls.run is base.Stencil.run and cls.verify_stencil is base.HorizontalDiffusionStencil.verify_stencil
    for cls in (vertical_advection.SharedMem, vertical_advection.Slab, vertical_advection.TensorMem,
                vertical_advection.GlobalScratch, vertical_advection.NoAlloc):
        assert issubclass(cls, base.VerticalAdvectionStencil)
        assert cls.verify_stencil is base.VerticalAdvectionStencil.verify_stencil
    assert issubclass(basic.Laplacian, base.LaplacianStencil) and issubclass(basic.Copy, base.CopyStencil)
    assert issubclass(basic.SymmetricAverage, base.SymmetricAverageStencil)
    # the reference's parameters, plus this backend's additions
    params = horizontal_diffusion.TmaTile.parameters
    assert {"domain", "data_sets", "halo", "dtype", "layout", "alignment", "huge_pages", "offset_allocations",
            "verify"} <= set(params)
    assert {"dry_runs", "timers", "gpu_architecture", "block_size", "compute_dtype", "autotune", "device"} <= set(params)
    assert params["alignment"].default == 64


def test_cli_tree_of_the_reference_holds_the_backend(ref):
    click = pytest.importorskip("click")
    from stencil_benchmarks_gb300 import cli as launcher

    ref_cli = launcher.prepare()
    benchmark = ref[0]
    group = ref_cli._build([(ref_cli._cli_command(b), ref_cli._cli_func(b)) for b in benchmark.REGISTRY])
    gb300 = group.commands["stencils"].commands["gb300"]
    assert isinstance(gb300, click.Group)
    assert set(gb300.commands["horizontal-diffusion"].commands) == {"j-scan", "tile", "tma-tile", "vector-scan"}
    assert set(gb300.commands["vertical-advection"].commands) == {"shared-mem", "global-scratch", "slab",
                                                                  "no-alloc", "tensor-mem"}
    assert "native" in group.commands["stream"].commands["gb300"].commands
    # the reference's own backends stay in the same tree
    assert "cuda-hip" in group.commands["stencils"].commands and "openmp" in group.commands["stencils"].commands
    names = {p.name for p in gb300.commands["horizontal-diffusion"].commands["tma-tile"].params}
    assert {"domain", "halo", "dtype", "verify", "block_size", "dry_runs", "timers", "autotune"} <= names


def test_construction_without_a_gpu_is_a_parameter_error(ref):
    """Without a GPU every gb300 benchmark refuses construction with the
    reference's ParameterError (the reference's CLI skips those with -s)."""
    from tests.conftest import gpu_available

    benchmark = ref[0]
    if gpu_available():
        pytest.skip("a GPU is present")
    ours = _ours(benchmark)
    assert len(ours) == 15
    for bmark in ours:
        with pytest.raises(benchmark.ParameterError):
            bmark()


def test_parameter_checks_come_before_allocation(ref):
    from stencil_benchmarks_gb300.benchmarks_collection.stencils.gb300 import horizontal_diffusion, vertical_advection

    benchmark = ref[0]
    with pytest.raises(benchmark.ParameterError, match="bfloat16"):
        horizontal_diffusion.JScan(dtype="bfloat16", domain=(8, 8, 2), halo=(2, 2, 0))
    with pytest.raises(benchmark.ParameterError, match="fixed64"):
        vertical_advection.SharedMem(compute_dtype="fixed64", domain=(8, 8, 2), halo=(1, 1, 0))
    with pytest.raises(benchmark.ParameterError, match="block_size"):
        horizontal_diffusion.TmaTile(block_size=(48, 4, 16), domain=(8, 8, 2), halo=(2, 2, 0))
    with pytest.raises(benchmark.ParameterError):
        horizontal_diffusion.TmaTile(timers="cpu")


def test_stdlib_report_modes(tmp_path, capsys):
    pytest.importorskip("click")
    from stencil_benchmarks_gb300 import cli as launcher

    rows = [{"time": t, "bandwidth": 1.0 / t, "domain": d, "dtype": "float64"}
            for d, t in (("(32, 32, 8)", 2.0), ("(32, 32, 8)", 4.0), ("(64, 32, 8)", 1.0))]
    out = tmp_path / "r.csv"
    launcher.stdlib_report(rows, {"time", "bandwidth"}, str(out), "all-medians")
    text = capsys.readouterr().out.splitlines()
    assert text[0].split() == ["domain", "time", "bandwidth"]
    assert text[1].split()[-2:] == ["1", "1"] and text[2].split()[-2] == "3"  # sorted by the median time
    assert len(out.read_text().splitlines()) == 4
    launcher.stdlib_report(rows, {"time", "bandwidth"}, None, "best-median")
    assert len(capsys.readouterr().out.splitlines()) == 2


def test_host_helper_equivalents(ref):
    """The stand-ins for the reference's compiled helpers give what its
    alloc_array and Stencil.random_field need: writable page-aligned buffers
    and a U[0, 1) fill."""
    from stencil_benchmarks.tools import array as ref_array

    from stencil_benchmarks_gb300 import host

    alloc = host._alloc_module()
    buf = alloc.alloc_smallpages(10000)
    assert isinstance(buf, mmap.mmap) and ctypes.addressof(ctypes.c_char.from_buffer(buf)) % mmap.PAGESIZE == 0
    assert alloc.l1_dcache_linesize() > 0
    a = ref_array.alloc_array((20, 10, 5), "float64", (2, 1, 0), 64, index_to_align=(2, 2, 0),
                              alloc=alloc.alloc_smallpages)
    host._parallel_module().random_fill(a)
    assert 0.0 <= a.min() and a.max() < 1.0 and a.std() > 0.1
    with pytest.raises(TypeError):
        host._parallel_module().random_fill(np.zeros(4, dtype=np.uint16))


@pytest.mark.parametrize("shape,dtype,layout,alignment,index", [
    ((2, 3), "int32", (1, 0), 0, None),
    ((2, 3), "int32", (0, 1), 64, None),
    ((20, 10, 5), "float64", (2, 1, 0), 128, (3, 3, 1)),
    ((516, 516, 80), "float64", (2, 1, 0), 64, (2, 2, 0)),
    ((33, 17, 9), "float32", (0, 1, 2), 32, (1, 1, 1)),
    ((33, 17, 9), "float32", (1, 2, 0), 0, (2, 2, 2)),
])
def test_array_layout_matches_the_reference(ref, shape, dtype, layout, alignment, index):
    """This package's host arrays (used where the reference is not loaded: the
    C-ABI tests, the bench) have the reference's strides and alignment."""
    from stencil_benchmarks.tools import array as ref_array

    want = ref_array.alloc_array(shape, dtype, layout, alignment, index_to_align=index)
    got = sbarray.alloc_array(shape, dtype, layout, alignment, index_to_align=index)
    assert got.strides == want.strides and got.shape == want.shape
    if alignment:
        idx = index or (0,) * len(shape)
        assert (got.ctypes.data + sum(s * i for s, i in zip(got.strides, idx))) % alignment == 0
    assert sbarray.nbytes(got) == ref_array.nbytes(want)


def test_bfloat16_arrays_hold_bit_patterns():
    assert sbarray.alloc_array((4, 4, 4), "bfloat16", (2, 1, 0)).dtype == np.uint16
