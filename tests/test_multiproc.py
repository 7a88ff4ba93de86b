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


def _shard_main(rank, world, port, out):
    """one rank of the row-block split: its block of A times the whole B (the CPU
    oracle stands in for the GPU), then the all-gather of per-shard entry counts
    that places the block in the global C"""
    import numpy as np
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from hsmu_gb import gen, shard

    A = gen.rmat(11, 16, seed=7)
    B = gen.poisson_random(A.N, 6, seed=8, ncols=5000)
    cuts = shard.row_blocks(A, B, world)
    blk = shard.host_block(A, int(cuts[rank]), int(cuts[rank + 1]))
    rp, col, val = oracle.spgemm(blk, B)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, torch.tensor([int(rp[-1])], dtype=torch.int64))
    offs = shard.global_offsets([int(c.item()) for c in counts])
    shards = [None] * world
    dist.all_gather_object(shards, (rp, col, val))
    out[rank] = (int(offs[rank]), shards if rank == 0 else None, cuts.tolist())
    dist.destroy_process_group()


def test_two_ranks_row_blocks_stitch_to_the_one_shot_product():
    pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp

    import oracle
    from hsmu_gb import gen, shard

    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_shard_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    res = dict(out)
    A = gen.rmat(11, 16, seed=7)
    B = gen.poisson_random(A.N, 6, seed=8, ncols=5000)
    rp, col, val = shard.stitch(res[0][1], B.N)
    want = oracle.spgemm(A, B)
    np.testing.assert_array_equal(rp, want[0])
    np.testing.assert_array_equal(col, want[1])
    assert np.array_equal(val.view(np.int64), want[2].view(np.int64))
    # rank 1's rows start where rank 0's entries end
    assert res[1][0] == int(res[0][1][0][0][-1])
    cuts = res[0][2]
    assert cuts[0] == 0 and cuts[-1] == A.M and cuts[0] < cuts[1] < cuts[2]


@pytest.mark.parametrize("parts", [1, 3, 8])
def test_row_blocks_balance_products(parts):
    import numpy as np

    from hsmu_gb import gen, shard

    A = gen.rmat(12, 16, seed=2)
    cuts = shard.row_blocks(A, A, parts)
    assert len(cuts) == parts + 1 and cuts[0] == 0 and cuts[-1] == A.M
    assert np.all(np.diff(cuts) >= 0)
    prod = shard.row_products(A, A)
    per = np.array([prod[cuts[r]:cuts[r + 1]].sum() for r in range(parts)])
    assert per.sum() == prod.sum()
    # each block is within one row's products of an equal share
    assert np.all(np.abs(per - prod.sum() / parts) <= prod.max() + 1)
