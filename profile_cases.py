"""Launch named kernel cases a fixed number of times (for ncu captures).

    python profile_cases.py [--warmup W] [--launches L] CASE...

CASE is ``<stencil>-<form>[:<variant>[@<placement>]]`` with stencil in hdiff, vadv, vadv3 (all
three components on a shared wcon, one launch each, or ``vadv3-<form>:fused`` for
the single sb_vadv3 launch), triad, copy, lap and
form in f64, f32, bf16 (bf16 = bfloat16 storage, f32 compute), f32x2
(float64 storage, float-pair compute) and fix64 (float64 storage, hdiff only,
fixed-point sums); ``all`` runs every hdiff/vadv form plus triad-f64.  Stencil cases use the 512 x 512 x 80
interior with the reference's halos (2 for hdiff, 1 for vadv); triad uses
2^27 elements.  Each case allocates its fields, runs W warm-up launches and L
measured launches (CUDA events), prints one line per case, and frees its
fields before the next case.  The kernel variants are the defaults of the
library, except vadv-f64 and vadv-f32x2, which use the caller-scratch
(GLOBAL) variant as ``bench.py`` does.  ``:<variant>`` picks another one
(hdiff: tile, jscan, tma, vscan -- tma with rows padded to 64 bytes so that the
j/k strides suit the tensor copies; vadv: smem, global, slab, wslab, tmem -- global,
slab and wslab with ccol/dcol scratch fields; lap: point, march); ``@<placement>``
sets the float64 integer-pipe placement preset (sb_tune.flags bits 4-7) of tma
(then on the library's default 128 x 4 tile, 16 rows, one k-plane per block: the
tile the presets apply to), slab and march.
"""

from __future__ import annotations

import argparse
import statistics
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

from stencil_benchmarks_gb300 import _native, kernels  # noqa: E402
from stencil_benchmarks_gb300 import array as sbarray  # noqa: E402
from stencil_benchmarks_gb300.device import DeviceBuffer, Field  # noqa: E402

NI, NJ, NK = 512, 512, 80
STORAGE = {"f64": ("float64", "float64"), "f32": ("float32", "float32"), "bf16": ("bfloat16", "float32"),
           "f32x2": ("float64", "float32x2"), "fix64": ("float64", "fixed64")}


def _field(rng, storage, halo, lo, hi, alignment=0):
    shape = (NI + 2 * halo[0], NJ + 2 * halo[1], NK + 2 * halo[2])
    host = sbarray.alloc_array(shape, storage, (2, 1, 0), alignment, index_to_align=halo)
    vals = rng.uniform(lo, hi, size=shape)
    if storage == "bfloat16":
        bits = vals.astype(np.float32).view(np.uint32).astype(np.uint64)
        host[...] = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
    else:
        host[...] = vals
    dev = Field.like_host(host, storage, halo)
    dev.upload(host)
    return dev


VARIANTS = {"tile": _native.HDIFF_TILE, "jscan": _native.HDIFF_JSCAN, "tma": _native.HDIFF_TMA,
            "vscan": _native.HDIFF_VSCAN,
            "smem": _native.VADV_SMEM, "wslab": _native.VADV_WSLAB, "tmem": _native.VADV_TMEM,
            "global": _native.VADV_GLOBAL, "slab": _native.VADV_SLAB,
            "point": _native.BASIC_POINT, "march": _native.BASIC_MARCH}


def run_case(name, warmup, launches, rng):
    name, _, variant = name.partition(":")
    variant, _, placement = variant.partition("@")
    flags = int(placement) << 4 if placement else 0
    stencil, form = name.split("-")
    if stencil == "triad":
        n = 1 << 27
        bufs = [DeviceBuffer(n * 8) for _ in range(3)]
        a, b, c = (x.ptr for x in bufs)
        kernels.stream_op(_native.STREAM_INIT, "float64", a, b, c, n)

        def launch(timed):
            return kernels.stream_op(_native.STREAM_TRIAD, "float64", a, b, c, n, 3.0, timed=timed)
    else:
        storage, compute = STORAGE[form]
        if stencil == "hdiff":
            align = 64 if variant == "tma" else 0
            f = [_field(rng, storage, (2, 2, 0), 0.0, 1.0, align) for _ in range(3)]

            htune = None
            if variant == "tma" and placement:
                htune = _native.tune(variant=VARIANTS[variant], block_x=128, block_y=4, tile_y=16, k_per_cta=1,
                                     flags=flags)
            elif variant:
                htune = _native.tune(variant=VARIANTS[variant], flags=flags)

            def launch(timed):
                return kernels.hdiff(*f, compute=compute, tune=htune, timed=timed)
        elif stencil == "vadv":
            f = [_field(rng, storage, (1, 1, 0), -1.0, 1.0) for _ in range(4)]
            f.append(_field(rng, storage, (1, 1, 0), -0.5, 0.5))
            out = _field(rng, storage, (1, 1, 0), 0.0, 0.0)
            scratch = {}
            tune = None
            scratch_storage = "float64" if compute in ("float64", "float32x2") else "float32"
            if variant in ("global", "slab", "wslab") or (not variant and form in ("f64", "f32x2")):
                scratch = {"ccol": _field(rng, scratch_storage, (1, 1, 0), 0.0, 0.0),
                           "dcol": _field(rng, scratch_storage, (1, 1, 0), 0.0, 0.0)}
            if variant == "slab":  # the bench's tunings for f64 and f32x2
                slab = {"f64": (32, 1, 0), "f32x2": (64, 2, 32)}.get(form, (64, 4, 16))
                tune = _native.tune(variant=_native.VADV_SLAB, block_x=slab[0], unroll=slab[1], k_per_cta=slab[2],
                                    flags=flags)
            elif variant:
                tune = _native.tune(variant=VARIANTS[variant])
            elif form in ("f64", "f32x2"):
                tune = _native.tune(variant=_native.VADV_GLOBAL, block_x=64 if form == "f64" else 32,
                                    unroll=2 if form == "f64" else 1)

            def launch(timed):
                return kernels.vadv(*f, out=out, compute=compute, tune=tune, timed=timed, **scratch)
        elif stencil == "vadv3":  # all components: u, v, w on one wcon field, three launches
            comps = [[_field(rng, storage, (1, 1, 1), -1.0, 1.0) for _ in range(4)] for _ in range(3)]
            wcon = _field(rng, storage, (1, 1, 1), -0.5, 0.5)
            outs = [_field(rng, storage, (1, 1, 1), 0.0, 0.0) for _ in range(3)]

            def launch(timed):
                if variant == "fused":  # one sb_vadv3 launch
                    return kernels.vadv3(comps, wcon, outs=outs, compute=compute, timed=timed)
                total = 0.0
                for f, o, shift in zip(comps, outs, ((1, 0), (0, 1), (0, 0))):
                    t = kernels.vadv(*f, wcon, shift, out=o, compute=compute, timed=timed)
                    total += t or 0.0
                return total
        elif stencil in ("copy", "lap"):
            f = [_field(rng, storage, (1, 1, 1), 0.0, 1.0) for _ in range(2)]
            ltune = _native.tune(variant=VARIANTS[variant], flags=flags) if variant else None

            def launch(timed):
                if stencil == "copy":
                    return kernels.copy(*f, timed=timed)
                return kernels.laplacian(*f, compute=compute, tune=ltune, timed=timed)
        else:
            raise SystemExit(f"unknown case {name!r}")
    for _ in range(warmup):
        launch(False)
    times = [launch(True) for _ in range(launches)]
    print(f"{name}: {launches} launches, median {statistics.median(times) * 1e6:.1f} us", flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("cases", nargs="+")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--launches", type=int, default=1)
    args = ap.parse_args(argv)
    cases = []
    for c in args.cases:
        if c == "all":
            cases += [f"{s}-{f}" for s in ("hdiff", "vadv") for f in STORAGE if (s, f) != ("vadv", "fix64")]
            cases.append("triad-f64")
        else:
            cases.append(c)
    _native.call("sb_set_device", 0)
    rng = np.random.Generator(np.random.PCG64(7))
    for c in cases:
        run_case(c, args.warmup, args.launches, rng)
    return 0


if __name__ == "__main__":
    sys.exit(main())
