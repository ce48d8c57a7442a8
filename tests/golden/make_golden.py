"""Generate the golden fixtures in this directory from the reference itself.

Run in a container where the reference (GridTools/stencil_benchmarks 0.11.0)
is available at ``/root/reference`` (override with ``SB_REFERENCE``):

    python tests/golden/make_golden.py

For every case the script builds a reference benchmark instance, replaces its
(unseeded) random fields by seeded arrays, calls the reference's own
``verify_stencil`` and records the array that the reference compares the output
field against (its ``validation.check_equality`` is wrapped to capture the
``expected`` argument).  For horizontal diffusion it also records what the
reference's numpy backend (``stencils.numpy.horizontal_diffusion.OnTheFly``)
writes.  Inputs and captured outputs go to ``<case>.npz``; the parameters go to
``cases.json``.

The reference's two pybind11 helpers (``tools.alloc`` for page-aligned host
buffers and ``tools.parallel`` for an unseeded random fill) are replaced by
small pure-Python stand-ins, because the fixtures only need seeded values and
plain host memory.  Nothing else of the reference is modified.
"""

from __future__ import annotations

import json
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("SB_REFERENCE", "/root/reference"))


def _import_reference():
    sys.path.insert(0, str(REFERENCE))
    alloc = types.ModuleType("stencil_benchmarks.tools.alloc")
    alloc.alloc_smallpages = lambda nbytes: bytearray(nbytes)
    alloc.alloc_hugepages = lambda nbytes, transparent=False: bytearray(nbytes)
    alloc.l1_dcache_linesize = lambda: 64
    alloc.l1_dcache_sets = lambda: 64
    parallel = types.ModuleType("stencil_benchmarks.tools.parallel")

    def random_fill(data):
        data[...] = 0

    parallel.random_fill = random_fill
    sys.modules["stencil_benchmarks.tools.alloc"] = alloc
    sys.modules["stencil_benchmarks.tools.parallel"] = parallel

    from stencil_benchmarks.benchmarks_collection.stencils import base
    from stencil_benchmarks.benchmarks_collection.stencils.numpy import (
        basic as np_basic,
    )
    from stencil_benchmarks.benchmarks_collection.stencils.numpy import (
        horizontal_diffusion as np_hdiff,
    )

    return base, np_basic, np_hdiff


def _capture(base):
    """Replace base.validation.check_equality by a recorder of (name, expected).

    The recorder never raises, so every field the reference would compare is
    captured (a raising check would stop at the first output)."""
    records = {}
    original = base.validation.check_equality

    def check_equality(name, result, expected):
        records[name] = np.array(expected, copy=True)

    base.validation.check_equality = check_equality
    return records, original


def _seeded(bench, seed, dists):
    """Seeded arrays with the benchmark's own shape/strides, one per arg."""
    rng = np.random.Generator(np.random.PCG64(seed))
    arrays = []
    for name in bench.args:
        field = bench.empty_field()
        low, high, quant = dists.get(name, dists.get("*", (0.0, 1.0, None)))
        values = rng.uniform(low, high, size=field.shape)
        if quant:
            values = np.round(values * quant) / quant
        field[...] = values.astype(field.dtype)
        arrays.append(field)
    return arrays


def main():
    base, np_basic, np_hdiff = _import_reference()

    class VAdv(base.VerticalAdvectionStencil):
        """Concrete reference vertical advection (its verify is the oracle)."""

        def run_stencil(self, data):
            return {"time": 1.0}

    class Hdiff(base.HorizontalDiffusionStencil):
        def run_stencil(self, data):
            return {"time": 1.0}

    vadv_dists = {
        "ustage": (-1.0, 1.0, None),
        "upos": (-1.0, 1.0, None),
        "utens": (-1.0, 1.0, None),
        "utensstage": (-1.0, 1.0, None),
        "vstage": (-1.0, 1.0, None),
        "vpos": (-1.0, 1.0, None),
        "vtens": (-1.0, 1.0, None),
        "vtensstage": (-1.0, 1.0, None),
        "wstage": (-1.0, 1.0, None),
        "wpos": (-1.0, 1.0, None),
        "wtens": (-1.0, 1.0, None),
        "wtensstage": (-1.0, 1.0, None),
        "wcon": (-0.5, 0.5, None),
        "*": (0.0, 1.0, None),
    }
    unit = {"*": (0.0, 1.0, None)}
    coarse = {"*": (0.0, 1.0, 8)}  # multiples of 1/8: ties in the limiter

    cases = [
        # name, kind, class, params, seed, dists, output fields
        ("hdiff_f64_h2", "hdiff", Hdiff, dict(domain=(16, 12, 5), halo=(2, 2, 0)), 11, unit),
        ("hdiff_f64_h3", "hdiff", Hdiff, dict(domain=(13, 7, 3), halo=(3, 3, 1)), 12, unit),
        ("hdiff_f32_h2", "hdiff", Hdiff,
         dict(domain=(16, 12, 4), halo=(2, 2, 0), dtype="float32"), 13, unit),
        ("hdiff_f64_ties", "hdiff", Hdiff, dict(domain=(10, 9, 2), halo=(2, 2, 0)), 14, coarse),
        ("vadv_f64", "vadv", VAdv, dict(domain=(12, 6, 9), halo=(1, 1, 0)), 21, vadv_dists),
        ("vadv_f32", "vadv", VAdv,
         dict(domain=(9, 5, 6), halo=(1, 1, 0), dtype="float32"), 22, vadv_dists),
        ("vadv_all_f64", "vadv", VAdv,
         dict(domain=(8, 7, 5), halo=(1, 1, 1), all_components=True), 23, vadv_dists),
        ("vadv_nk2_f64", "vadv", VAdv, dict(domain=(5, 4, 2), halo=(1, 1, 0)), 24, vadv_dists),
        ("copy_f64", "copy", np_basic.Copy, dict(domain=(10, 6, 4)), 31, unit),
        ("lap_xy_f64", "laplacian", np_basic.Laplacian,
         dict(domain=(10, 6, 4), halo=(1, 1, 1)), 32, unit),
        ("lap_xyz_f32", "laplacian", np_basic.Laplacian,
         dict(domain=(10, 6, 4), halo=(1, 1, 1), along_z=True, dtype="float32"), 33, unit),
        ("avg1_x_f64", "onesided_average", np_basic.OnesidedAverage,
         dict(domain=(10, 6, 4), halo=(1, 1, 1), axis=0), 34, unit),
        ("avg1_z_f64", "onesided_average", np_basic.OnesidedAverage,
         dict(domain=(10, 6, 4), halo=(1, 1, 1), axis=2), 35, unit),
        ("avg2_y_f64", "symmetric_average", np_basic.SymmetricAverage,
         dict(domain=(10, 6, 4), halo=(1, 1, 1), axis=1), 36, unit),
    ]

    meta = {}
    for name, kind, cls, params, seed, dists in cases:
        bench = cls(verify=True, **params)
        arrays = _seeded(bench, seed, dists)
        data_type = type(bench._data[0])
        before = data_type._make(np.array(a, copy=True) for a in arrays)
        # give "after" the expected outputs later; start from a copy
        after = data_type._make(np.array(a, copy=True) for a in arrays)
        records, original = _capture(base)
        try:
            try:
                bench.verify_stencil(before, after)
            except Exception:  # noqa: BLE001 - after.out is not the answer yet
                pass
        finally:
            base.validation.check_equality = original
        out_names = [n for n in records if n in ("out", "utensstage", "vtensstage", "wtensstage")]
        payload = {f"in_{n}": np.ascontiguousarray(a) for n, a in zip(bench.args, arrays)}
        for n in out_names:
            payload[f"expected_{n}"] = np.ascontiguousarray(records[n])
        if kind == "hdiff":
            # the reference's numpy backend on the same inputs
            numpy_backend = np_hdiff.OnTheFly(verify=False, **params)
            fields = data_type._make(np.array(a, copy=True) for a in arrays)
            numpy_backend.run_stencil(fields)
            sl = tuple(slice(h, h + d) for d, h in zip(bench.domain, bench.halo))
            payload["numpy_backend_out"] = np.ascontiguousarray(fields.out[sl])
        np.savez_compressed(HERE / f"{name}.npz", **payload)
        meta[name] = {
            "kind": kind,
            "seed": seed,
            "domain": list(bench.domain),
            "halo": list(bench.halo),
            "dtype": bench.dtype,
            "args": list(bench.args),
            "outputs": out_names,
            "params": {k: v for k, v in params.items() if k not in ("domain", "halo", "dtype")},
            "reference_class": f"{cls.__module__}.{cls.__name__}",
        }
        print(f"{name}: {', '.join(out_names)}")

    # STREAM: value of a, b, c after ntimes rounds (stream/cuda_hip.j2:329-345)
    stream = {}
    for dtype in ("float64", "float32"):
        t = np.dtype(dtype).type
        for ntimes in (1, 2, 10):
            aj, bj, cj, s = t(1), t(2), t(0), t(3)
            for _ in range(ntimes):
                cj = aj
                bj = s * cj
                cj = aj + bj
                aj = bj + s * cj
            stream[f"{dtype}_{ntimes}"] = [float(aj), float(bj), float(cj)]
    meta["_stream_scalars"] = stream

    (HERE / "cases.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
