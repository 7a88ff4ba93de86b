"""bench.py's multi-rank plumbing (one process per GPU: replicas of the product,
barrier before and after the timed region, the step time taken as the max over
ranks) on two CPU processes with the gloo backend."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    bench.dist_barrier(world)
    out[rank] = bench.dist_max(1.5 + rank, world)  # every rank must see the slowest rank's time
    bench.dist_barrier(world)
    dist.destroy_process_group()


def test_two_ranks_barrier_and_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}
