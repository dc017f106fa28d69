"""Host-side logic of bench.py, on CPU: the multi-rank timing reduction over
gloo (world size 2), the job-throughput arithmetic, and the reference arm's
JSON line (which needs no GPU)."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist()
    try:
        slowest = d.max(1.0 + rank)  # rank 1 is the slow one
        d.barrier()
        q.put((rank, slowest, bench.job_rate(1000, slowest, d.world)))
    finally:
        d.close()


def test_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    # both ranks see the slowest rank's time; the job rate counts both ranks' units
    assert got == [(0, 2.0, 1000.0), (1, 2.0, 1000.0)]


def test_job_rate_is_whole_job_throughput():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_rate(10, 2.0, 1) == 5.0
    assert bench.job_rate(10, 2.0, 4) == 20.0


def test_reference_arm_prints_one_json_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "histo",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "GUP/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["n_gpus"] == 1 and d["warmup"] >= 3


@pytest.mark.parametrize("world", [2])
def test_reference_arm_under_torchrun_prints_once(world):
    port = 30500 + (os.getpid() % 1000)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={world}",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--workload", "histo", "--steps", "1", "--warmup", "3",
                        "--gpus", str(world)], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["n_gpus"] == world
