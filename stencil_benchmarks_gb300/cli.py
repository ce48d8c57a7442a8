"""``sbench``-style command line for the GB300 backend.

Same command tree and options as the reference's CLI
(stencil_benchmarks/cli.py:47-245): every registered benchmark becomes
``<module path after the package's first two components> <kebab-case class>``,
e.g. ``stencils gb300 horizontal-diffusion j-scan``; each Parameter becomes an
option (booleans as ``--flag/--no-flag``); global options ``-e/--executions``,
``-r/--report``, ``-s/--skip-invalid-parameters``,
``-q/--skip-execution-failures`` and ``-o/--output`` (CSV).  Parameter values
may be lists in brackets, ``--domain [256,512] 512 80``, which run the
cartesian product.  Exit status 1 on an execution error, 2 on a validation
error, as in the reference.  The report is printed with the standard library
(the reference uses pandas).

    python -m stencil_benchmarks_gb300.cli stencils gb300 horizontal-diffusion j-scan --domain 512 512 80
"""

from __future__ import annotations

import csv
import gc
import itertools
import re
import statistics
import sys
import types

import click

from . import benchmark, benchmarks_collection  # noqa: F401  (registers the benchmarks)
from .validation import ValidationError


def command_path(bmark):
    path = bmark.__module__.split(".")[2:]
    name = re.sub("(?!^)([A-Z1-9]+)", r"-\1", bmark.__name__).lower()
    return path + [name]


class ListOf(click.ParamType):
    """A value or a bracketed comma list of values of ``base``."""

    name = "value-or-list"

    def __init__(self, base):
        self.base = base

    def convert(self, value, param, ctx):
        if isinstance(value, list):
            return value
        text = str(value)
        if text.startswith("[") and text.endswith("]"):
            return [self.base(v.strip()) for v in text[1:-1].split(",") if v.strip()]
        return [self.base(text)]


def _parse_scalar(dtype):
    if dtype is bool:
        return lambda v: v if isinstance(v, bool) else str(v).lower() in ("1", "true", "yes")
    return dtype


def _options(bmark):
    for name, param in bmark.parameters.items():
        flag = "--" + name.replace("_", "-")
        help_text = param.description[0].upper() + param.description[1:] + "."
        if param.dtype is bool:
            yield click.option(flag + "/" + flag.replace("--", "--no-"), default=param.default, help=help_text,
                               show_default=True)
        else:
            yield click.option(flag, type=ListOf(_parse_scalar(param.dtype)), nargs=param.nargs,
                               required=param.default is None, default=param.default, help=help_text,
                               show_default=param.default is not None)


def _expand(kwargs):
    """Cartesian product over every option given as a list."""
    keys, choices = [], []
    for key, value in kwargs.items():
        if value is None:
            continue
        if isinstance(value, tuple) and value and isinstance(value[0], list):
            combos = [tuple(c) for c in itertools.product(*value)]
        elif isinstance(value, list):
            combos = value
        else:
            combos = [value]
        keys.append(key)
        choices.append(combos)
    for combo in itertools.product(*choices):
        yield dict(zip(keys, combo))


def _report(results, output, report):
    if not results:
        click.echo("no data collected")
        sys.exit(1)
    if output:
        with open(output, "w", newline="") as fh:
            writer = csv.DictWriter(fh, fieldnames=list(results[0]))
            writer.writeheader()
            writer.writerows(results)
    numeric = [k for k, v in results[0].items() if isinstance(v, (int, float)) and not isinstance(v, bool)]
    keys = [k for k in results[0] if k not in numeric]
    varying = [k for k in keys if len({str(r[k]) for r in results}) > 1]
    if report == "full":
        for r in results:
            click.echo("  ".join(f"{k}={r[k]}" for k in r))
        return
    groups = {}
    for r in results:
        groups.setdefault(tuple(str(r[k]) for k in varying), []).append(r)
    rows = []
    for gkey, rs in groups.items():
        med = {k: statistics.median(float(r[k]) for r in rs) for k in numeric}
        rows.append((gkey, med))
    rows.sort(key=lambda x: x[1].get("time", 0.0))
    if report == "best-median":
        rows = rows[:1]
    header = varying + numeric
    click.echo("  ".join(f"{h:>14}" for h in header))
    for gkey, med in rows:
        click.echo("  ".join([f"{v:>14}" for v in gkey] + [f"{med[k]:>14.6g}" for k in numeric]))


def _command(bmark):
    @click.pass_context
    def func(ctx, **kwargs):
        results = []
        for kws in _expand(kwargs):
            try:
                instance = bmark(**kws)
            except benchmark.ParameterError as err:
                if ctx.obj.skip_invalid_parameters:
                    continue
                click.echo(*err.args)
                sys.exit(1)
            for _ in range(ctx.obj.executions):
                try:
                    out = instance.run()
                except benchmark.ExecutionError as err:
                    if ctx.obj.skip_execution_failures:
                        continue
                    click.echo("\nexecution error: " + " ".join(str(a) for a in err.args).strip())
                    sys.exit(1)
                except ValidationError as err:
                    click.echo("\nvalidation error: " + " ".join(str(a) for a in err.args).strip())
                    sys.exit(2)
                for r in out if isinstance(out, list) else [out]:
                    row = {k: (str(v) if isinstance(v, (tuple, list)) else v) for k, v in instance.parameters.items()}
                    row.update(r)
                    results.append(row)
            del instance
            gc.collect()
        _report(results, ctx.obj.output, ctx.obj.report)

    for option in _options(bmark):
        func = option(func)
    return func


@click.group()
@click.option("--executions", "-e", type=int, default=3)
@click.option("--report", "-r", default="all-medians", type=click.Choice(["best-median", "all-medians", "full"]))
@click.option("--skip-invalid-parameters", "-s", is_flag=True)
@click.option("--skip-execution-failures", "-q", is_flag=True)
@click.option("--output", "-o", type=click.Path())
@click.pass_context
def _root(ctx, executions, report, skip_invalid_parameters, skip_execution_failures, output):
    ctx.obj.executions = executions
    ctx.obj.report = report
    ctx.obj.skip_invalid_parameters = skip_invalid_parameters
    ctx.obj.skip_execution_failures = skip_execution_failures
    ctx.obj.output = output


def build_group():
    tree = {}
    for bmark in benchmark.REGISTRY:
        if not bmark.__module__.startswith(__package__ + "."):
            continue
        path = command_path(bmark)
        node = tree
        for part in path[:-1]:
            node = node.setdefault(part, {})
        node[path[-1]] = bmark

    def attach(group, subtree):
        for name, sub in sorted(subtree.items()):
            if isinstance(sub, dict):

                @click.pass_context
                def empty(_):
                    pass

                attach(group.group(name=name.replace("_", "-"))(empty), sub)
            else:
                group.command(name=name)(_command(sub))

    root = click.Group(name="sbench-gb300", callback=_root.callback, params=list(_root.params))
    attach(root, tree)
    return root


def main(*args, **kwargs):
    return build_group()(*args, **kwargs, obj=types.SimpleNamespace())


if __name__ == "__main__":
    main()
