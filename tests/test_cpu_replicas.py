"""Replica path of bench.py under torch.distributed (gloo, world size 2, CPU).

A single scene does not shard (no halo exchange in the reference), so N GPUs run N
replicas: every rank times its own frames, the max over ranks is the job time and
the summed particle-substeps over that time is the value. These tests run the
timing reduction and the barrier on two CPU ranks, and the replica arithmetic with
the CPU oracle standing in for each rank's step.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    r, w, lr = bench.dist_env()
    assert (r, w, lr) == (rank, world, rank)
    # each rank steps its own replica (the oracle stands in for the GPU step) and times it
    import time

    import oracle as O
    from helpers import config_for, make_pair, small_pile

    sc = small_pile(4)
    _, orc = make_pair(sc, config_for(sc), gpu=False)
    t0 = time.perf_counter()
    for _ in range(2 + rank):  # unequal work: the job time is the slowest rank's
        orc.step(1.0 / 60.0, 2, 1)
    mine = time.perf_counter() - t0
    bench.barrier(world)
    job = bench.reduce_max(mine, world)
    out[rank] = (mine, job)
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    mine = [out[r][0] for r in range(world)]
    job = [out[r][1] for r in range(world)]
    assert job[0] == job[1] == max(mine)
