"""The host framework this backend plugs into: the reference's own
``stencil_benchmarks`` package.

The GB300 benchmark classes are subclasses of the reference's
``stencil_benchmarks.benchmark.Benchmark`` and of its ``Stencil`` base classes
(stencil_benchmarks/benchmarks_collection/stencils/base.py:45-501), so they
enter the reference's ``REGISTRY`` (stencil_benchmarks/benchmark.py:140-164),
appear in its CLI tree (stencil_benchmarks/cli.py:47-50) and are run and
verified by the reference's ``Stencil.run`` / ``verify_stencil``.

``load()`` makes the package importable and returns it.  It looks for

1. an importable ``stencil_benchmarks`` (site-packages, ``PYTHONPATH``);
2. ``$SBGB300_REFERENCE``, a directory holding the package;
3. ``baseline/_ref`` at the repository root, the copy that
   ``__graft_entry__.build()`` installs from the reference's sources.

The package has two compiled pybind11 helpers: ``tools.alloc`` (page-aligned
host buffers and the L1 cache geometry) and ``tools.parallel`` (an unseeded
multithreaded U[0, 1) fill).  A copy installed on one machine and used on
another architecture has neither loadable; ``load()`` then registers
equivalents written here (mmap-backed page-aligned buffers, the geometry
from sysfs, a numpy fill with the same distribution) before anything imports
them.  Nothing else of the package is replaced.
"""

from __future__ import annotations

import importlib
import mmap
import os
import sys
import types
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent
DEFAULT_COPY = REPO / "baseline" / "_ref"

_loaded = None
#: names of the compiled helpers replaced by the equivalents below
replaced_helpers: list = []


class HostFrameworkMissing(ImportError):
    """The reference's ``stencil_benchmarks`` package cannot be found."""


def _sysfs_int(path: str, default: int) -> int:
    try:
        with open(path) as f:
            return int(f.read().strip().rstrip("K"))
    except (OSError, ValueError):
        return default


def _alloc_module():
    mod = types.ModuleType("stencil_benchmarks.tools.alloc")

    def alloc_smallpages(size):
        buf = mmap.mmap(-1, max(int(size), 1), flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
        if hasattr(mmap, "MADV_NOHUGEPAGE"):
            buf.madvise(mmap.MADV_NOHUGEPAGE)
        return buf

    def alloc_hugepages(size, transparent):
        huge = _sysfs_int("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", 2 << 20)
        paged = (max(int(size), 1) + huge - 1) // huge * huge
        flags = mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS
        if not transparent:
            flags |= getattr(mmap, "MAP_HUGETLB", 0x40000)
        try:
            buf = mmap.mmap(-1, paged, flags=flags)
        except OSError as err:
            raise MemoryError(f"huge-page allocation of {paged} bytes failed: {err}") from err
        if transparent and hasattr(mmap, "MADV_HUGEPAGE"):
            buf.madvise(mmap.MADV_HUGEPAGE)
        return buf

    cache = "/sys/devices/system/cpu/cpu0/cache/index0/"
    mod.alloc_smallpages = alloc_smallpages
    mod.alloc_hugepages = alloc_hugepages
    mod.l1_dcache_linesize = lambda: _sysfs_int(cache + "coherency_line_size", 64)
    mod.l1_dcache_sets = lambda: _sysfs_int(cache + "number_of_sets", 0)
    return mod


def _parallel_module():
    mod = types.ModuleType("stencil_benchmarks.tools.parallel")
    rng = np.random.default_rng()

    def random_fill(data):
        if not np.issubdtype(data.dtype, np.floating):
            raise TypeError(f"random_fill: unsupported element type {data.dtype}")
        data[...] = rng.random(data.shape, dtype=np.float64).astype(data.dtype)

    mod.random_fill = random_fill
    return mod


def _install_helpers():
    for name, make in (("alloc", _alloc_module), ("parallel", _parallel_module)):
        full = f"stencil_benchmarks.tools.{name}"
        try:
            importlib.import_module(full)
        except ImportError:
            sys.modules[full] = make()
            setattr(sys.modules["stencil_benchmarks.tools"], name, sys.modules[full])
            replaced_helpers.append(name)


def _candidates():
    env = os.environ.get("SBGB300_REFERENCE")
    if env:
        yield Path(env)
    yield DEFAULT_COPY


def load():
    """Import the reference's ``stencil_benchmarks`` package and return it."""
    global _loaded
    if _loaded is not None:
        return _loaded
    try:
        pkg = importlib.import_module("stencil_benchmarks")
    except ImportError:
        pkg = None
        for path in _candidates():
            if (path / "stencil_benchmarks" / "__init__.py").is_file():
                sys.path.insert(0, str(path))
                pkg = importlib.import_module("stencil_benchmarks")
                break
        if pkg is None:
            raise HostFrameworkMissing(
                "the stencil_benchmarks package (GridTools/stencil_benchmarks) is not importable: install it, "
                "set SBGB300_REFERENCE to a directory that holds it, or run __graft_entry__.build() where its "
                "sources are available to install a copy under baseline/_ref"
            ) from None
    importlib.import_module("stencil_benchmarks.tools")
    _install_helpers()
    _loaded = pkg
    return pkg


def install_copy(source: Path, target: Path = DEFAULT_COPY) -> bool:
    """Install the reference package from its sources into ``target`` with pip.

    The sources are copied to a temporary directory first (pip builds in the
    source tree and the sources may be read-only); dependencies come from the
    machine, except ``click``, which the package imports and which is
    installed beside it when a wheel of it can be found offline
    (``$PIP_FIND_LINKS``).  Returns False when ``target`` already holds the
    package."""
    import shutil
    import subprocess
    import tempfile

    if (target / "stencil_benchmarks" / "__init__.py").is_file():
        return False
    target.mkdir(parents=True, exist_ok=True)
    pip = [sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation", "--no-deps",
           "--target", str(target), "--quiet"]
    links = os.environ.get("PIP_FIND_LINKS")
    if links:
        pip += ["--find-links", links]
    with tempfile.TemporaryDirectory() as tmp:
        src = Path(tmp) / "src"
        shutil.copytree(source, src, ignore=shutil.ignore_patterns(".git", "build", "*.egg-info"))
        subprocess.run(pip + [str(src)], check=True, cwd=tmp)
    if links:
        subprocess.run(pip + ["click"], check=False)
    return True


def available() -> bool:
    try:
        load()
        return True
    except ImportError:
        return False
