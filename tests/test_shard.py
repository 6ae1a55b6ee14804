"""Splitting a batch of independent t-SNE systems over ranks (CPU, gloo).

The batch has no exchange step: each rank owns whole systems.  These tests
check the split (a partition, deterministic, balanced by particle count) and
the two host-side collectives a multi-rank run uses (MAX of elapsed times,
SUM of processed particles) on two gloo ranks.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from masterthesislucas_gb300 import shard


def _sizes(count=256, seed=2024):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(2000), np.log(200000), count)).astype(np.int64)


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_assign_is_a_balanced_partition(world):
    sizes = _sizes()
    owned = shard.assign(sizes, world)
    flat = sorted(i for o in owned for i in o)
    assert flat == list(range(len(sizes)))
    loads = np.array([sizes[o].sum() for o in owned])
    # greedy LPT: the spread is at most the largest single system
    assert loads.max() - loads.min() <= sizes.max()
    assert owned == shard.assign(sizes, world)
    for r in range(world):
        assert shard.shard(sizes, r, world) == owned[r]


def test_assign_edge_cases():
    assert shard.assign([], 2) == [[], []]
    assert shard.assign([5], 3) == [[0], [], []]
    # equal sizes go round-robin from rank 0
    assert shard.assign([7, 7, 7, 7], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.assign([1, 2], 0)
    with pytest.raises(ValueError):
        shard.assign([1, -2], 2)
    with pytest.raises(ValueError):
        shard.shard([1, 2], 2, 2)


def test_single_process_collectives_are_identity():
    assert shard.max_over_ranks(1.25) == 1.25
    assert shard.sum_over_ranks(17) == 17


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = _sizes()
        mine = shard.shard(sizes, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        elapsed = 0.5 + rank  # rank 1 is the slow one
        t = shard.max_over_ranks(elapsed)
        total = shard.sum_over_ranks(int(sizes[mine].sum()))
        out.put((rank, gathered, t, total))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_and_reduce():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    results = [out.get() for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sizes = _sizes()
    for rank, gathered, t, total in results:
        assert gathered == shard.assign(sizes, world)
        assert t == 1.5
        assert total == int(sizes.sum())
