"""The multi-GPU path is replicas only (independent lines, no exchange step):
its host-side logic -- max-over-ranks timing, the whole-job rate, rank-only
work in the reference arm -- on world_size-2 gloo process groups on CPU."""
from __future__ import annotations

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, ws, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=ws)
    t = bench.max_over_ranks(torch, 10.0 + 5.0 * rank, "cpu")
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ws = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, join=True, start_method="spawn")
    assert dict(out) == {0: 15.0, 1: 15.0}


def test_whole_job_rate_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.whole_job_rate(1, 20, 8, 1 << 20, 100.0)
    assert bench.whole_job_rate(4, 20, 8, 1 << 20, 100.0) == pytest.approx(4 * one)
    assert one == pytest.approx(20 * 8 * (1 << 20) / 0.1)


def test_reference_arm_other_ranks_do_nothing():
    """Under torchrun only rank 0 of the reference arm runs and prints."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       timeout=120, env=env, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""
