"""Autotuner for the batched launch (replaces the reference's manual
block-size sweeps, stencil_benchmarks/tools/multirun.py:75-92 and the
scripts/sbench_*_collection.py configurations).

``autotune_batch`` times every candidate launch shape -- threads per hdiff
block, persistent hdiff blocks per SM (the rest of each SM is left to the
vadv kernels running beside them), rows per hdiff work item, columns per vadv
block, and which kernels enter the graph first -- on the batch it is given (a few graph replays each, CUDA events, median)
and returns the fastest.  Results are cached in a JSON file keyed by GPU
name, storage/compute form and a coarse signature of the workload (number of
hdiff and vadv domains, total points and the largest nk, each rounded to a
power of two), so a recurring workload is tuned once.

Cache file: ``$SBGB300_TUNE_CACHE`` or ``~/.cache/sbgb300/autotune.json``.
"""

from __future__ import annotations

import json
import math
import os
import statistics
from pathlib import Path
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

from . import _native
from .batching import Batch, Domain, HdiffDomain

DEFAULT_CANDIDATES: List[Dict[str, int]] = [
    {"block": b, "blocks_per_sm": p, "hdiff_rows": r, "hdiff_planes": pl, "vadv_block": vb, "vadv_blocks_per_sm": vp,
     "order": o}
    for b in (128, 256)
    for p in (2, 4, 8)
    for r in (32, 64)
    for pl in (1, 2)
    for vb in (32, 64)
    for vp in (0, 2)
    for o in (0, 1)
    if b * p <= 2048 and (o == 0 or (vb == 32 and vp == 0 and p >= 4))
]


def cache_path() -> Path:
    env = os.environ.get("SBGB300_TUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "sbgb300" / "autotune.json"


def _pow2(x: float) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(1.0, x)))))


def signature(domains: Sequence[Domain]) -> str:
    nh = sum(isinstance(d, HdiffDomain) for d in domains)
    nv = len(domains) - nh
    pts, max_nk = 0, 0
    for d in domains:
        f = d.inp if isinstance(d, HdiffDomain) else d.stage
        ni, nj, nk = (n - 2 * h for n, h in zip(f.shape, f.halo))
        pts += ni * nj * nk
        max_nk = max(max_nk, nk)
    return f"h{_pow2(nh)}-v{_pow2(nv)}-p{_pow2(pts)}-k{_pow2(max_nk)}"


def _load_cache(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(path: Path, data: dict) -> None:
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home just means no cache


def time_batch(batch: Batch, reps: int = 3, warmup: int = 1, stream=None) -> float:
    for _ in range(warmup):
        batch.launch(stream)
    return statistics.median(batch.launch(stream, timed=True) for _ in range(reps))


def autotune_batch(storage: str, domains: Sequence[Domain], max_nk: int, compute: Optional[str] = None,
                   candidates: Optional[Iterable[Dict[str, int]]] = None, reps: int = 3, use_cache: bool = True,
                   ) -> Tuple[Dict[str, int], List[Tuple[float, Dict[str, int]]]]:
    """Return (best parameters, [(seconds, parameters), ...] of every candidate timed).

    With a cache hit the list is empty and no kernel runs."""
    compute = compute or ("float64" if storage == "float64" else "float32")
    key = "|".join([_native.device_info(_native.current_device())["name"], storage, compute, signature(domains)])
    path = cache_path()
    cache = _load_cache(path) if use_cache else {}
    if use_cache and key in cache:
        return dict(cache[key]["params"]), []
    results = []
    for params in list(candidates or DEFAULT_CANDIDATES):
        batch = None
        try:
            batch = Batch(storage, compute, max_domains=max(1, len(domains)), max_nk=max_nk, **params)
            batch.set(domains)
            t = time_batch(batch, reps=reps)
        except _native.SbError:
            continue
        finally:
            if batch is not None:
                batch.close()
        results.append((t, dict(params)))
    if not results:
        raise RuntimeError("no batch configuration could be launched")
    results.sort(key=lambda r: r[0])
    best = results[0][1]
    if use_cache:
        cache[key] = {"params": best, "seconds": results[0][0]}
        _store_cache(path, cache)
    return best, results
