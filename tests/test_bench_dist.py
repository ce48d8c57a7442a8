"""The multi-rank side of bench.py on the CPU (gloo, world size 2): the
max-over-ranks timing, the barrier, and the reference arm under torchrun
(rank 0 alone runs and prints one JSON line; the other rank exits 0)."""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    dist = bench.Dist()
    dist.barrier()
    value = dist.max(float(10 * rank + 1))
    dist.barrier()
    dist.close()
    Path(out_dir, f"rank{rank}.txt").write_text(repr(value))


def test_max_over_ranks_with_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)] == [11.0, 11.0]


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    from oracle import cport

    cport.build()  # the C restatement, the reference arm's fallback
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3"]
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                         env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # the reference's own OpenMP backends when its package loads and compiles here, else the C port
    from stencil_benchmarks_gb300 import host

    assert line["cpu_baseline"]["kind"] == ("reference" if host.available() else "port")
    assert line["config"] == {"workload": "hdiff+vadv fp64 512x512x80 (halo 2,2,0 / 1,1,0)",
                              "l2": "inputs > L2 (1.35 GB of fields per step), no flush"}
    assert not (ROOT / "benchmarks_source_code").exists(), "the reference's generated sources landed in the checkout"
