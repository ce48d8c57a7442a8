"""Build ``libsbgb300.so`` in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel to an object in
``_build/`` and linked into ``stencil_benchmarks_gb300/libsbgb300.so`` (static
CUDA runtime, so the library only needs the driver at run time).  Objects are
rebuilt when their source or any header changed.

    python -m stencil_benchmarks_gb300.build [--force] [--verbose]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIBRARY = PKG / "libsbgb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--fmad=false",  # one rounding per operation, like numpy; fma only where written
    "-Xcompiler",
    "-fPIC,-O2",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    mtime = obj.stat().st_mtime
    return mtime < src.stat().st_mtime or mtime < newest_header


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = _sources()
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    flags = list(NVCC_FLAGS) + list(extra_flags or [])
    jobs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        if force or _stale(obj, src, newest_header):
            cmd = [nvcc(), *ARCH, *flags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        return src, res

    failed = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as pool:
        for src, res in pool.map(run, jobs):
            out = (res.stdout + res.stderr).strip()
            if res.returncode != 0:
                failed.append(f"{src.name}:\n{out}")
            elif verbose and out:
                print(out)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))

    objs = [BUILD / (s.stem + ".o") for s in sources]
    newest_obj = max(o.stat().st_mtime for o in objs)
    if force or jobs or not LIBRARY.exists() or LIBRARY.stat().st_mtime < newest_obj:
        tmp = LIBRARY.with_name(f".{LIBRARY.name}.{os.getpid()}.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
        os.replace(tmp, LIBRARY)
    return LIBRARY


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args(argv)
    path = build(force=args.force, verbose=args.verbose)
    print(path)


if __name__ == "__main__":
    sys.exit(main())
