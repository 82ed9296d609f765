"""bench.py's multi-process plumbing on the CPU (gloo, world size 2).

The path does not shard across GPUs (one capture is one GPU's work): `bench.py --gpus N` runs N
replicas, one process per GPU, whose only collectives are the barrier around the timed region
and the max-over-ranks reduction of its time. Those two, and the reference arm's rank-0-only
rule under torchrun, are tested here without a GPU.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, _ = bench.dist_env()
    dist = bench.init_dist(w, "gloo")
    bench.barrier(dist)
    seconds = 1.0 + r            # each rank's "timed region"
    worst = bench.max_over_ranks(seconds, dist)
    bench.barrier(dist)
    Path(out, f"rank{r}.json").write_text(json.dumps({"rank": r, "world": w, "max": worst}))
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_with_gloo(tmp_path: Path) -> None:
    import torch.multiprocessing as mp

    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    results = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert [d["rank"] for d in results] == [0, 1]
    assert all(d["world"] == 2 and d["max"] == 2.0 for d in results)


def test_single_process_needs_no_process_group() -> None:
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.init_dist(1, "gloo") is None
    assert bench.max_over_ranks(3.5, None) == 3.5
    bench.barrier(None)


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once(tmp_path: Path) -> None:
    port = free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    proc = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
         "--impl", "reference", "--gpus", "2", "--workload", "fir63", "--steps", "1",
         "--warmup", "0"],
        capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [l for l in proc.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                     # rank 0 alone runs and prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
