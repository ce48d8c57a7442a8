"""The side-by-side harness's summary (reference_gpu.py): per stencil and
dtype, each side's fastest verified case, or its fastest unverified one,
marked, when none passed; STREAM by triad bandwidth.  No GPU needed."""

from __future__ import annotations

import reference_gpu


def _row(stencil, impl, cls, ms, verified=True, dtype="float64"):
    return {"stencil": stencil, "dtype": dtype, "impl": impl, "class": cls, "ms": ms,
            "gpoints_per_s": 1.0 / ms, "domain": [8, 8, 8], "verified": verified}


def test_fastest_verified_case_per_side():
    rows = [_row("hdiff", "reference cuda_hip", "A", 2.0), _row("hdiff", "reference cuda_hip", "B", 1.0, "fails"),
            _row("hdiff", "reference cuda_hip", "C", 1.5), _row("hdiff", "gb300", "X", 0.5),
            _row("hdiff", "gb300", "Y", 0.4, "fails")]
    (entry,) = reference_gpu.summary(rows)
    assert entry["reference"]["class"] == "C" and entry["reference"]["verified"]
    assert entry["gb300"]["class"] == "X"
    assert abs(entry["speedup"] - 3.0) < 1e-12


def test_unverified_side_is_reported_as_such():
    rows = [_row("vadv", "reference cuda_hip", "A", 2.0, "fails", "float32"),
            _row("vadv", "reference cuda_hip", "B", 1.0, "fails", "float32"),
            _row("vadv", "gb300", "X", 0.5, dtype="float32")]
    (entry,) = reference_gpu.summary(rows)
    assert entry["reference"]["class"] == "B" and entry["reference"]["verified"] is False
    assert entry["gb300"]["verified"] is True


def test_errors_are_skipped_and_stream_compares_triad():
    rows = [{"stencil": "vadv", "dtype": "float64", "impl": "gb300", "class": "Z", "error": "boom"},
            {"stencil": "stream", "dtype": "float64", "impl": "reference cuda_hip", "class": "Native",
             "params": {"vector_size": 1}, "gbs": {"triad": 5000.0}},
            {"stencil": "stream", "dtype": "float64", "impl": "reference cuda_hip", "class": "Native",
             "params": {"vector_size": 2}, "gbs": {"triad": 7000.0}},
            {"stencil": "stream", "dtype": "float64", "impl": "gb300", "class": "Native", "params": {},
             "gbs": {"triad": 7300.0}}]
    (entry,) = reference_gpu.summary(rows)
    assert entry["stencil"] == "stream"
    assert entry["reference"]["triad_gbs"] == 7000.0
    assert abs(entry["speedup"] - 7300.0 / 7000.0) < 1e-12
