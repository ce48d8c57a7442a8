"""Command tree of the CLI and the bridge to the reference's verification."""

from __future__ import annotations

import collections
import os
import sys
import types
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from tests.conftest import golden_cases, load_golden

REFERENCE = Path(os.environ.get("SB_REFERENCE", "/root/reference"))


def test_cli_command_tree():
    click = pytest.importorskip("click")
    from stencil_benchmarks_gb300 import cli

    group = cli.build_group()
    assert isinstance(group, click.Group)
    stencils = group.commands["stencils"].commands["gb300"]
    assert set(stencils.commands) >= {"basic", "horizontal-diffusion", "vertical-advection"}
    assert set(stencils.commands["horizontal-diffusion"].commands) == {"j-scan", "tile", "tma-tile", "vector-scan"}
    assert set(stencils.commands["vertical-advection"].commands) == {"shared-mem", "global-scratch", "slab", "no-alloc",
                                                                     "tensor-mem"}
    assert set(stencils.commands["basic"].commands) >= {"copy", "laplacian", "onesided-average",
                                                        "symmetric-average"}
    assert "native" in group.commands["stream"].commands["gb300"].commands
    # every parameter is an option
    jscan = stencils.commands["horizontal-diffusion"].commands["j-scan"]
    names = {p.name for p in jscan.params}
    assert {"domain", "halo", "dtype", "verify", "block_size", "dry_runs", "timers"} <= names


def test_cli_list_expansion():
    pytest.importorskip("click")
    from stencil_benchmarks_gb300 import cli

    combos = list(cli._expand({"domain": ([256, 512], [512], [80]), "dtype": ["float32", "float64"], "x": None}))
    assert len(combos) == 4
    assert {"domain": (256, 512, 80), "dtype": "float32"} in combos


def _import_reference():
    if not REFERENCE.exists():
        pytest.skip("reference not available here")
    sys.path.insert(0, str(REFERENCE))
    alloc = types.ModuleType("stencil_benchmarks.tools.alloc")
    alloc.alloc_smallpages = lambda n: bytearray(n)
    alloc.alloc_hugepages = lambda n, t=False: bytearray(n)
    alloc.l1_dcache_linesize = lambda: 64
    alloc.l1_dcache_sets = lambda: 64
    parallel = types.ModuleType("stencil_benchmarks.tools.parallel")
    parallel.random_fill = lambda a: a.__setitem__(Ellipsis, 0)
    sys.modules.setdefault("stencil_benchmarks.tools.alloc", alloc)
    sys.modules.setdefault("stencil_benchmarks.tools.parallel", parallel)


def _fake_stencil(meta):
    domain, halo = tuple(meta["domain"]), tuple(meta["halo"])

    def inner_slice(shift=None, expand=None):
        shift = shift if shift is not None else (0, 0, 0)
        return tuple(slice(h + s, h + d + s) for d, h, s in zip(domain, halo, shift))

    params = dict(meta["params"])
    for key, default in (("all_components", False), ("along_x", True), ("along_y", True), ("along_z", False)):
        params.setdefault(key, default)
    return SimpleNamespace(domain=domain, halo=halo, dtype=meta["dtype"], inner_slice=inner_slice, **params)


@pytest.mark.parametrize("name", ["hdiff_f64_h2", "vadv_all_f64", "lap_xyz_f32"])
def test_reference_bridge_verifies_with_the_reference(name):
    _import_reference()
    from stencil_benchmarks_gb300 import reference_bridge, validation, verification

    saved = verification.registered()
    try:
        assert reference_bridge.install()
        meta = golden_cases()[name]
        data = load_golden(name)
        kind = {"hdiff": "horizontal_diffusion", "vadv": "vertical_advection"}.get(meta["kind"], meta["kind"])
        stencil = _fake_stencil(meta)
        fields = {n: np.array(data[f"in_{n}"]) for n in meta["args"]}
        data_t = collections.namedtuple("StencilData", meta["args"])
        before = data_t(**{n: a.copy() for n, a in fields.items()})
        after = data_t(**{n: a.copy() for n, a in fields.items()})
        sl = stencil.inner_slice()
        for out in meta["outputs"]:
            getattr(after, out)[sl] = data[f"expected_{out}"]
        verification.get(kind)(stencil, before, after)  # correct answer passes
        getattr(after, meta["outputs"][0])[sl][0, 0, 0] += 1.0
        before = data_t(**{n: a.copy() for n, a in fields.items()})
        with pytest.raises(validation.ValidationError):
            verification.get(kind)(stencil, before, after)
    finally:
        for k in list(verification.registered()):
            verification.unregister(k)
        for k, fn in saved.items():
            verification.register(k, fn)
