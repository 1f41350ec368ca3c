"""The bench's multi-GPU logic on the CPU: replicas on every rank, the whole-job value from the
slowest rank's time (max over ranks, here over two gloo processes), and the reference arm run by
rank 0 alone."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    t = bench.max_over_ranks(1.0 + rank, dist, device="cpu")
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}  # both ranks report the slowest rank's time


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank starts the reference arm; only rank 0 runs the CPU model and
    prints; the others exit 0 at once without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
