"""Scaling collection for GB300: ``sbench-gb300-collection``.

Counterpart of the reference's per-GPU collection scripts
(stencil_benchmarks/scripts/sbench_h100_collection.py, driven by
stencil_benchmarks/tools/multirun.py:43-92; its "stream" row is the halo-free
copy, as there): every configuration of a group
runs on the cubic-ish domains 32x32x80, 64x64x80, ..., 1024x1024x80
(``--min-exp``/``--max-exp`` change the range), ``--executions`` times each,
and every execution becomes one CSV row holding the configuration name, all
benchmark parameters and the result columns.  The table is written with the
standard library: the reference's driver (tools/multirun.py) imports pandas
at module level, which neither machine here has.

    python -m stencil_benchmarks_gb300.collection basic-bandwidth out.csv -e 11
    python -m stencil_benchmarks_gb300.collection horizontal-diffusion-bandwidth out.csv -o dtype='"float32"'

``-o name=value`` overrides a keyword of every configuration of the group
(value as a Python literal), as in the reference.
"""

from __future__ import annotations

import argparse
import ast
import csv
import gc
import re
import warnings
from typing import Callable, Dict, Iterable, List, Optional, Sequence, Tuple

from .benchmarks_collection.stencils.gb300 import basic, horizontal_diffusion as hdiff, vertical_advection as vadv
from .host import load

load()
from stencil_benchmarks.benchmark import ParameterError  # noqa: E402


class Configuration:
    """One named benchmark setup of a scaling run."""

    def __init__(self, ctor, name: Optional[str] = None, **kwargs):
        self.ctor = ctor
        self.name = name or re.sub("(?!^)([A-Z1-9]+)", r"-\1", ctor.__name__).lower()
        self.kwargs = kwargs

    def instantiate(self, domain, preprocess: Optional[Callable[..., Dict]] = None):
        kwargs = dict(self.kwargs, domain=domain)
        if preprocess is not None:
            kwargs = preprocess(**kwargs)
        return self.ctor(**kwargs)


def domains(min_exp: int = 5, max_exp: int = 11, k: int = 80) -> Iterable[Tuple[int, int, int]]:
    """(2^e, 2^e, k) for min_exp <= e < max_exp."""
    for e in range(min_exp, max_exp):
        yield 2**e, 2**e, k


def _row(name: str, instance, result: Dict) -> Dict:
    row = {"name": name}
    for key, value in instance.parameters.items():
        row[key] = str(value) if isinstance(value, (tuple, list)) else value
    row.update(result)
    return row


def run_scaling_benchmark(configurations: Sequence[Configuration], executions: int,
                          domain_range: Optional[Iterable[Tuple[int, int, int]]] = None,
                          preprocess: Optional[Callable[..., Dict]] = None, echo=print) -> List[Dict]:
    """Rows of every execution of every configuration on every domain."""
    rows: List[Dict] = []
    domain_range = list(domains() if domain_range is None else domain_range)
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        for domain in domain_range:
            for config in configurations:
                try:
                    instance = config.instantiate(domain, preprocess)
                except ParameterError as err:
                    echo(f"skipping {config.name} on {domain}: {err}")
                    continue
                for _ in range(executions):
                    out = instance.run()
                    for r in out if isinstance(out, list) else [out]:
                        rows.append(_row(config.name, instance, r))
                echo(f"{config.name} {domain[0]}x{domain[1]}x{domain[2]}: {executions} executions")
                del instance
                gc.collect()
    for message in sorted({str(w.message) for w in caught}):
        echo("WARNING: " + message)
    return rows


def write_csv(rows: Sequence[Dict], path: str) -> None:
    """All rows in one table; columns are the union of the rows' keys."""
    columns: List[str] = []
    for r in rows:
        columns += [k for k in r if k not in columns]
    with open(path, "w", newline="") as fh:
        writer = csv.DictWriter(fh, fieldnames=columns)
        writer.writeheader()
        writer.writerows(rows)


def common_kwargs(options: Sequence[str], **defaults):
    kwargs = dict(verify=False, dry_runs=1, **defaults)
    for option in options:
        name, value = option.split("=", 1)
        kwargs[name.replace("-", "_")] = ast.literal_eval(value)
    return kwargs


def _group_basic(kwargs):
    k3 = dict(kwargs, halo=(1, 1, 1))
    return [
        Configuration(basic.Copy, name="stream", **dict(kwargs, halo=(0, 0, 0))),
        Configuration(basic.Empty, name="empty", **k3),
        Configuration(basic.Copy, name="copy", **k3),
        Configuration(basic.OnesidedAverage, name="avg-i", axis=0, **k3),
        Configuration(basic.OnesidedAverage, name="avg-j", axis=1, **k3),
        Configuration(basic.OnesidedAverage, name="avg-k", axis=2, **k3),
        Configuration(basic.SymmetricAverage, name="sym-avg-i", axis=0, **k3),
        Configuration(basic.SymmetricAverage, name="sym-avg-j", axis=1, **k3),
        Configuration(basic.SymmetricAverage, name="sym-avg-k", axis=2, **k3),
        Configuration(basic.Laplacian, name="lap-ij", along_x=True, along_y=True, along_z=False, **k3),
    ]


def _group_hdiff(kwargs):
    k = dict(kwargs, halo=(2, 2, 0))
    return [
        Configuration(hdiff.JScan, **k),
        Configuration(hdiff.Tile, **k),
        Configuration(hdiff.TmaTile, **k),
        Configuration(hdiff.VectorScan, **k),
    ]


def _group_vadv(kwargs):
    k = dict(kwargs, halo=(1, 1, 0))
    configs = [Configuration(vadv.SharedMem, **k), Configuration(vadv.GlobalScratch, **k),
               Configuration(vadv.Slab, **k)]
    if kwargs.get("dtype", "float64") in ("float32", "bfloat16"):
        configs.append(Configuration(vadv.TensorMem, **k))
    return configs


GROUPS = {
    "basic-bandwidth": _group_basic,
    "horizontal-diffusion-bandwidth": _group_hdiff,
    "vertical-advection-bandwidth": _group_vadv,
}


def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(prog="sbench-gb300-collection",
                                 description="GB300 scaling collections (domains 32^2..1024^2 x 80).")
    sub = ap.add_subparsers(dest="group", required=True)
    for name in GROUPS:
        sp = sub.add_parser(name)
        sp.add_argument("output", help="CSV file to write")
        sp.add_argument("--executions", "-e", type=int, default=101)
        sp.add_argument("--option", "-o", action="append", default=[], help="name=value override (Python literal)")
        sp.add_argument("--min-exp", type=int, default=5, help="smallest domain 2^min_exp")
        sp.add_argument("--max-exp", type=int, default=11, help="largest domain 2^(max_exp-1)")
        sp.add_argument("--levels", type=int, default=80, help="k extent of every domain")
    args = ap.parse_args(argv)
    kwargs = common_kwargs(args.option, dtype="float64")
    # the kernels guard their own bounds: no block-size truncation for small
    # domains (the reference needs one for its generated code)
    rows = run_scaling_benchmark(GROUPS[args.group](kwargs), args.executions,
                                 domains(args.min_exp, args.max_exp, args.levels))
    write_csv(rows, args.output)
    print(f"{len(rows)} rows -> {args.output}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
