"""Precision report: hdiff and vadv at 512 x 512 x 80 in every storage /
compute form, on identical seeded inputs, against the float64 oracle.

Inputs: hdiff inp and coeff uniform in [0, 1); vadv stage, pos, tens and
tensstage uniform in [-1, 1), wcon uniform in [-0.5, 0.5) (wcon shifted by
+1 in i, the u component); one seed for all forms.  Each form stores the
float64 draws in its storage type (round to nearest), computes on the GPU and
is compared with the float64 oracle evaluated on the float64 draws:

  err_max_scale  max |got - oracle| / max |oracle|
  err_rms        rms(got - oracle) / rms(oracle)
  err_max_point  max |got - oracle| / |oracle| over points with
                 |oracle| >= 1e-3 max |oracle|
  err_point_pXX  percentiles of |got - oracle| / |oracle| over points with
                 |oracle| >= 1e-2 rms(oracle)
and, for the quantised forms, the same against the oracle evaluated in the
form's compute type on the form's own (quantised) inputs (the arithmetic
error alone).  hdiff's flux limiter is a discontinuity: quantised inputs
flip some limiter decisions, and each flip moves its outputs by a whole
flux, so hdiff also reports the oracle's decisions that sit exactly on the
zero boundary (ties), how many decisions the quantised form takes the other
way, and the errors over the outputs that no flipped decision feeds.
Throughput: median CUDA-event kernel time over `reps` launches, compulsory
bytes / time and grid points / time.

Conditioning: with wcon uniform in [-0.5, 0.5) and dtr_stage = 3/20 the
vadv diagonal bcol = 0.15 - acol - ccol ranges over [-0.1, 0.4], so some
columns are close to singular (results far above the inputs' magnitude).
Their error dominates the max-norm columns of every form, including the
float32-stored inputs on their own; the percentiles show the typical point.

    python -m tests.precision_report [--size NI NJ NK] [--reps R] [--json PATH]

The oracle and this script are test infrastructure (not the product path).
"""

from __future__ import annotations

import argparse
import json
import statistics
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import stencils as ora  # noqa: E402
from stencil_benchmarks_gb300 import _native, kernels  # noqa: E402
from tests.gpu_helpers import as_compute, download_like, host_field, interior, to_device  # noqa: E402

HDIFF_FORMS = [("float64", "float64"), ("float64", "fixed64"), ("float64", "float32x2"), ("float32", "float64"),
               ("float32", "float32"), ("bfloat16", "float32")]
VADV_FORMS = [("float64", "float64"), ("float64", "float32x2"), ("float32", "float64"), ("float32", "float32"),
              ("bfloat16", "float32")]
ITEMSIZE = {"float64": 8, "float32": 4, "bfloat16": 2}


def _errors(got, ref, skip=None):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    d = np.abs(got - ref)
    scale = float(np.max(np.abs(ref)))
    big = np.abs(ref) >= 1e-3 * scale
    rms = float(np.sqrt(np.mean(ref * ref)))
    sig = np.abs(ref) >= 1e-2 * rms
    rel = d[sig] / np.abs(ref[sig])
    out = {
        "err_max_scale": float(d.max() / scale),
        "err_rms": float(np.sqrt(np.mean(d * d)) / rms),
        "err_max_point": float(np.max(d[big] / np.abs(ref[big]))),
        "err_point_p50": float(np.percentile(rel, 50)),
        "err_point_p99": float(np.percentile(rel, 99)),
        "err_point_p999": float(np.percentile(rel, 99.9)),
        "scale": scale, "rms": rms,
    }
    if skip is not None:  # outputs fed by a limiter decision that differs from the oracle's
        keep = ~skip
        out["points_with_flipped_limiter"] = int(np.count_nonzero(skip))
        out["err_max_scale_unflipped"] = float(d[keep].max() / scale) if keep.any() else 0.0
        out["err_max_point_unflipped"] = float(np.max(d[keep & big] / np.abs(ref[keep & big])))
    return out


def _affected(flips_x, flips_y):
    """Interior outputs that use a flipped flux: flx(i), flx(i-1), fly(j), fly(j-1)."""
    return flips_x[1:] | flips_x[:-1] | flips_y[:, 1:] | flips_y[:, :-1]


def _limited(inp, domain, halo):
    """Limiter decisions (True = flux set to 0) of the fluxes feeding the interior:
    flx for i = -1 .. ni-1 (shape ni+1, nj, nk), fly for j = -1 .. nj-1."""
    hi, hj, _ = halo
    ni, nj, _ = domain
    sl = ora.inner_slice(domain, halo)
    lap = np.zeros_like(inp)
    lap[1:-1, 1:-1, :] = 4 * inp[1:-1, 1:-1, :] - (
        inp[2:, 1:-1, :] + inp[:-2, 1:-1, :] + inp[1:-1, 2:, :] + inp[1:-1, :-2, :])
    fx, fxp = (slice(hi - 1, hi + ni), sl[1], sl[2]), (slice(hi, hi + ni + 1), sl[1], sl[2])
    fy, fyp = (sl[0], slice(hj - 1, hj + nj), sl[2]), (sl[0], slice(hj, hj + nj + 1), sl[2])
    return ((lap[fxp] - lap[fx]) * (inp[fxp] - inp[fx]) > 0,
            (lap[fyp] - lap[fy]) * (inp[fyp] - inp[fy]) > 0)


def _time(launch, reps):
    launch(False)
    launch(False)
    return statistics.median(launch(True) for _ in range(reps))


def hdiff_report(domain, reps, seed=2024):
    halo = (2, 2, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(seed))
    vals = {"inp": rng.uniform(0.0, 1.0, size=shape), "coeff": rng.uniform(0.0, 1.0, size=shape)}
    ref = ora.hdiff(vals["inp"], vals["coeff"], domain, halo)
    ties, total = ora.hdiff_limiter_stats(vals["inp"], vals["coeff"], domain, halo)
    ref_lim = _limited(vals["inp"], domain, halo)
    points = int(np.prod(domain))
    rows = []
    for storage, compute in HDIFF_FORMS:
        hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
        hosts["out"] = host_field(np.zeros(shape), storage, halo=halo)
        dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}

        def launch(timed):
            return kernels.hdiff(dev["inp"], dev["coeff"], dev["out"], compute=compute, timed=timed)

        t = _time(launch, reps)
        got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
        if storage == "bfloat16":
            got = ora.bf16_bits_to_f32(np.ascontiguousarray(got)).reshape(got.shape)
        skip = None
        if storage != "float64":
            # the kernel's own decisions: the form's compute type on its stored inputs
            cdt = np.float32 if compute == "float32" else np.float64
            qin = {n: as_compute(hosts[n], storage).astype(cdt) for n in ("inp", "coeff")}
            q_lim = _limited(qin["inp"], domain, halo)
            flips = [a != b for a, b in zip(ref_lim, q_lim)]
            skip = _affected(*flips)
        row = {"stencil": "hdiff", "storage": storage, "compute": compute, **_errors(got, ref, skip)}
        if storage != "float64":
            qref = ora.hdiff(qin["inp"], qin["coeff"], domain, halo)
            row["vs_oracle_on_quantised_inputs"] = _errors(got, qref)
            row["limiter_flips_from_quantisation"] = int(sum(np.count_nonzero(f) for f in flips))
        nbytes = ITEMSIZE[storage] * ((domain[0] + 4) * (domain[1] + 4) * domain[2] + 2 * points)
        row.update(time_us=t * 1e6, gpoints_s=points / t / 1e9, bytes_moved=nbytes, hbm_gbs=nbytes / t / 1e9)
        rows.append(row)
        del dev
    return {"limiter_ties_exact_zero": ties, "limiter_decisions": total, "forms": rows}


def vadv_report(domain, reps, seed=2025):
    halo = (1, 1, 0)
    shape = tuple(d + 2 * h for d, h in zip(domain, halo))
    rng = np.random.Generator(np.random.PCG64(seed))
    names = ("stage", "pos", "tens", "tensstage", "wcon")
    vals = {n: rng.uniform(-1.0, 1.0, size=shape) for n in names[:4]}
    vals["wcon"] = rng.uniform(-0.5, 0.5, size=shape)
    ref = ora._vadv_component(*[vals[n] for n in names], domain, halo, 1, 0)
    points = int(np.prod(domain))
    rows = []
    for storage, compute in VADV_FORMS:
        hosts = {n: host_field(v, storage, halo=halo) for n, v in vals.items()}
        hosts["out"] = host_field(np.zeros(shape), storage, halo=halo)
        dev = {n: to_device(h, storage, halo) for n, h in hosts.items()}
        scratch_type = "float64" if compute in ("float64", "float32x2") else "float32"
        scratch = {n: to_device(host_field(np.zeros(shape), scratch_type, halo=halo), scratch_type, halo)
                   for n in ("ccol", "dcol")}
        tune = None
        if compute in ("float64", "float32x2") and storage == "float64":
            tune = _native.tune(variant=_native.VADV_SLAB, block_x=64, unroll=2 if compute == "float32x2" else 4,
                                k_per_cta=32 if compute == "float32x2" else 8)

        def launch(timed):
            return kernels.vadv(*[dev[n] for n in names], (1, 0), out=dev["out"], compute=compute, tune=tune,
                                timed=timed, **(scratch if tune is not None else {}))

        t = _time(launch, reps)
        got = interior(download_like(dev["out"], hosts["out"]), domain, halo)
        if storage == "bfloat16":
            got = ora.bf16_bits_to_f32(np.ascontiguousarray(got)).reshape(got.shape)
        row = {"stencil": "vadv", "storage": storage, "compute": compute, **_errors(got, ref)}
        if storage != "float64":
            cdt = np.float32 if compute == "float32" else np.float64
            qin = [as_compute(hosts[n], storage).astype(cdt) for n in names]
            qref = ora._vadv_component(*qin, domain, halo, 1, 0)
            row["vs_oracle_on_quantised_inputs"] = _errors(got, qref)
        nbytes = ITEMSIZE[storage] * (5 * points + (domain[0] + 1) * domain[1] * domain[2])
        row.update(time_us=t * 1e6, gpoints_s=points / t / 1e9, bytes_moved=nbytes, hbm_gbs=nbytes / t / 1e9)
        rows.append(row)
        del dev, scratch
    return {"forms": rows}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--size", type=int, nargs=3, default=(512, 512, 80))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--json", type=Path, default=None)
    args = ap.parse_args(argv)
    _native.call("sb_set_device", 0)
    domain = tuple(args.size)
    report = {"domain": domain, "hdiff": hdiff_report(domain, args.reps), "vadv": vadv_report(domain, args.reps)}
    text = json.dumps(report, indent=1)
    if args.json:
        args.json.write_text(text)
    for section in ("hdiff", "vadv"):
        for r in report[section]["forms"]:
            q = r.get("vs_oracle_on_quantised_inputs", {})
            print(f"{section:5s} {r['storage']:8s}/{r['compute']:9s} max(scale) {r['err_max_scale']:.2e} "
                  f"[unflipped {r.get('err_max_scale_unflipped', r['err_max_scale']):.2e}] "
                  f"rms {r['err_rms']:.2e} p99 {r['err_point_p99']:.2e} p99.9 {r['err_point_p999']:.2e} "
                  f"max(point) {r['err_max_point']:.2e} | arith-only max(scale) "
                  f"{q.get('err_max_scale', float('nan')):.2e} | {r['time_us']:8.1f} us "
                  f"{r['gpoints_s']:7.1f} GPts/s {r['hbm_gbs']:7.1f} GB/s", flush=True)
    h = report["hdiff"]
    print(f"hdiff limiter ties at exact zero: {h['limiter_ties_exact_zero']} of {h['limiter_decisions']}; "
          f"flips from quantisation: " + ", ".join(f"{r['storage']}: {r['limiter_flips_from_quantisation']}"
                                                  for r in h["forms"] if "limiter_flips_from_quantisation" in r))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
