"""Multi-rank logic of bench.py on CPU (gloo, world size 2): the replica
throughput takes the slowest rank's time and all ranks' bytes; the reference
arm's non-zero ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    dist.barrier()
    ms, value = bench.replica_throughput(10.0 + 5.0 * rank, step_bytes=1_000_000, steps=4, world=world,
                                         device="cpu")
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_replica_throughput_max_over_ranks_gloo():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 15.0                              # the slower rank
        assert value == pytest.approx(1_000_000 * 4 * world / 0.015 / 1e9)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.replica_throughput(2.0, step_bytes=10 ** 9, steps=1, world=1, device="cpu")
    assert ms == 2.0 and value == pytest.approx(500.0)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
