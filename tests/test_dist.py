"""The multi-rank partition of the path on CPU: two gloo ranks split a quartet list, reduce a
J-like sum and a timing, and reproduce the single-process result."""
import os

import numpy as np
import pytest

from libcint_gb300.dist import balanced_order, rank_slice


def test_rank_slices_cover_once():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [rank_slice(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_balanced_order_lpt():
    costs = [10, 1, 1, 1, 9, 2, 2]
    owner = balanced_order(costs, 2)
    loads = [sum(c for c, o in zip(costs, owner) if o == r) for r in range(2)]
    assert abs(loads[0] - loads[1]) <= 2


def _worker(rank, world, port, result):
    import torch
    import torch.distributed as dist
    from libcint_gb300.dist import max_over_ranks, shard, sum_over_ranks
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    rng = np.random.RandomState(0)
    items = np.arange(1000)
    vals = rng.normal(size=(1000, 5))
    mine = shard(items, rank, world)
    acc = torch.tensor(vals[mine].sum(0))
    sum_over_ranks(acc)
    t = max_over_ranks(1.0 + rank)
    result[rank] = (acc.numpy().tolist(), t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_one_process():
    import torch.multiprocessing as mp
    pytest.importorskip('torch.distributed')
    port = 29500 + os.getpid() % 2000
    mgr = mp.Manager()
    result = mgr.dict()
    mp.spawn(_worker, args=(2, port, result), nprocs=2, join=True)
    rng = np.random.RandomState(0)
    vals = rng.normal(size=(1000, 5))
    for r in range(2):
        acc, t = result[r]
        np.testing.assert_allclose(acc, vals.sum(0), rtol=1e-12, atol=1e-12)
        assert t == 2.0
