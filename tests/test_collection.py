"""Scaling collection driver: configuration names, domain range, option
overrides and the CSV table (CPU parts); one small sweep on the GPU."""

from __future__ import annotations

import csv

import pytest

from stencil_benchmarks_gb300 import collection
from stencil_benchmarks_gb300.benchmarks_collection.stencils.gb300 import horizontal_diffusion as hdiff


def test_domains_match_the_reference_range():
    assert list(collection.domains()) == [(32, 32, 80), (64, 64, 80), (128, 128, 80), (256, 256, 80),
                                          (512, 512, 80), (1024, 1024, 80)]
    assert list(collection.domains(6, 8, 40)) == [(64, 64, 40), (128, 128, 40)]


def test_configuration_names_and_overrides():
    assert collection.Configuration(hdiff.JScan).name == "j-scan"
    assert collection.Configuration(hdiff.TmaTile).name == "tma-tile"
    kw = collection.common_kwargs(["dtype='float32'", "alignment=128"], dtype="float64")
    assert kw["dtype"] == "float32" and kw["alignment"] == 128 and kw["verify"] is False


def test_groups_cover_every_gb300_form():
    names = {c.name for c in collection.GROUPS["horizontal-diffusion-bandwidth"]({})}
    assert names == {"j-scan", "tile", "tma-tile", "vector-scan"}
    assert "tensor-mem" in {c.name for c in collection.GROUPS["vertical-advection-bandwidth"]({"dtype": "float32"})}
    assert "tensor-mem" not in {c.name for c in collection.GROUPS["vertical-advection-bandwidth"]({})}
    basic = [c.name for c in collection.GROUPS["basic-bandwidth"]({})]
    assert basic[0] == "stream" and "lap-ij" in basic


def test_csv_has_the_union_of_columns(tmp_path):
    rows = [{"name": "a", "time": 1.0}, {"name": "b", "time": 2.0, "bandwidth": 3.0}]
    out = tmp_path / "t.csv"
    collection.write_csv(rows, str(out))
    got = list(csv.DictReader(open(out)))
    assert [r["name"] for r in got] == ["a", "b"] and got[0]["bandwidth"] == "" and got[1]["bandwidth"] == "3.0"


@pytest.mark.gpu
def test_small_sweep_on_the_gpu(tmp_path, lib):
    rows = collection.run_scaling_benchmark(collection.GROUPS["horizontal-diffusion-bandwidth"]({"dtype": "float32"}),
                                            2, collection.domains(5, 7, 16), echo=lambda *_: None)
    assert len(rows) == 4 * 2 * 2 and all(r["time"] > 0 for r in rows)
    out = tmp_path / "h.csv"
    collection.write_csv(rows, str(out))
    assert len(list(csv.DictReader(open(out)))) == 16


def test_main_parses_groups_and_options(tmp_path, monkeypatch):
    seen = {}

    def fake_run(configs, executions, domain_range, **_):
        seen["names"] = [c.name for c in configs]
        seen["executions"] = executions
        seen["domains"] = list(domain_range)
        seen["dtype"] = configs[0].kwargs["dtype"]
        return [{"name": "x", "time": 1.0}]

    monkeypatch.setattr(collection, "run_scaling_benchmark", fake_run)
    out = tmp_path / "v.csv"
    assert collection.main(["vertical-advection-bandwidth", str(out), "-e", "2", "--min-exp", "6", "--max-exp", "7",
                            "-o", "dtype='float32'"]) == 0
    assert seen == {"names": ["shared-mem", "global-scratch", "slab", "tensor-mem"], "executions": 2,
                    "domains": [(64, 64, 80)], "dtype": "float32"}
    assert out.exists()
