"""``sbench`` with the GB300 backend registered.

A launcher over the reference's own CLI (stencil_benchmarks/cli.py:241-245),
as the reference's ``scripts/sbench.py:34-38`` is: it loads the reference's
``stencil_benchmarks`` package (``host.load()``), imports the reference's
benchmark collection and this backend's, so that every class is in the
reference's ``REGISTRY``, and calls ``stencil_benchmarks.cli.main``.  The
command tree, options, range syntax (``--domain [256,512] 512 80``), exit
codes and ``-e/-r/-s/-q/-o`` are the reference's.

The reference prints its report with pandas (``_process_results``,
stencil_benchmarks/cli.py:86-116).  Where pandas is not installed the
launcher puts a standard-library report with the same three modes
(``full``, ``all-medians``, ``best-median``) and the same CSV option in its
place; with pandas present nothing is replaced.

    python -m stencil_benchmarks_gb300.cli stencils gb300 horizontal-diffusion tma-tile --domain 512 512 80
"""

from __future__ import annotations

import csv
import importlib.util
import statistics
import sys

from .host import load


def stdlib_report(results, result_keys, output, report):
    """The reference's ``_process_results`` contract without pandas."""
    import click

    if not results:
        click.echo("no data collected")
        sys.exit(1)
    columns = list(dict.fromkeys(k for r in results for k in r))
    if output:
        with open(output, "w", newline="") as fh:
            writer = csv.DictWriter(fh, fieldnames=columns)
            writer.writeheader()
            writer.writerows(results)

    def is_num(k):
        return all(isinstance(r.get(k), (int, float)) and not isinstance(r.get(k), bool) for r in results)

    numeric = [k for k in columns if k in result_keys and is_num(k)]
    varying = [k for k in columns if k not in numeric and len({repr(r.get(k)) for r in results}) > 1]
    if report == "full":
        shown = [k for k in columns if k in numeric or k in varying]
        click.echo("  ".join(f"{k:>14}" for k in shown))
        for r in results:
            click.echo("  ".join(f"{r.get(k)!s:>14}" for k in shown))
        return
    groups = {}
    for r in results:
        groups.setdefault(tuple(repr(r.get(k)) for k in varying), []).append(r)
    rows = [(key, {k: statistics.median(float(r[k]) for r in rs) for k in numeric}) for key, rs in groups.items()]
    rows.sort(key=lambda row: row[1].get("time", 0.0))
    if report == "best-median":
        rows = rows[:1]
    click.echo("  ".join(f"{h:>14}" for h in varying + numeric))
    for key, med in rows:
        click.echo("  ".join([f"{v:>14}" for v in key] + [f"{med[k]:>14.6g}" for k in numeric]))


def prepare():
    """Load the reference, register both collections; return its cli module."""
    load()
    import stencil_benchmarks.benchmarks_collection  # noqa: F401
    from stencil_benchmarks import cli as ref_cli

    from . import benchmarks_collection  # noqa: F401

    if importlib.util.find_spec("pandas") is None:
        ref_cli._process_results = stdlib_report
    return ref_cli


def main(*args, **kwargs):
    return prepare().main(*args, **kwargs)


if __name__ == "__main__":
    main()
