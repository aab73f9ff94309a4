"""Multi-GPU is replicas only: each rank renders its own frames with its own seeds and the
benchmark combines them as (slowest rank's time, every rank's rays). Checked on CPU with two
gloo ranks; the reference arm runs on rank 0 alone."""
from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, rays = bench.replica_totals(10.0 * (rank + 1), 1000 * (rank + 1), "cpu")
    if rank == 0:
        Path(out).write_text(f"{ms} {rays}")
    dist.barrier()
    dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp

    out = tmp_path / "totals.txt"
    mp.spawn(_rank, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    ms, rays = out.read_text().split()
    assert float(ms) == 20.0 and int(rays) == 3000


def test_replica_totals_single_process():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_totals(12.5, 77, "cpu") == (12.5, 77)


def test_reference_arm_prints_only_on_rank_zero():
    """bench.py --impl reference under torchrun: ranks other than 0 exit 0 without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
