"""The multi-rank partition of the path on CPU: two gloo ranks split a quartet list, reduce a
J-like sum and a timing, and reproduce the single-process result; two gloo ranks shard the unique
quartet list by cost, contract their shares into J and K with the kernels' scheme (oracle blocks
standing in for each rank's GPU) and sum them into the full-tensor J and K."""
import os

import numpy as np
import pytest

from libcint_gb300 import molecules as M
from libcint_gb300.dist import balanced_order, rank_slice


def test_rank_slices_cover_once():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [rank_slice(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_balanced_order():
    costs = [10, 1, 1, 1, 9, 2, 2]
    owner = balanced_order(costs, 2)
    loads = [sum(c for c, o in zip(costs, owner) if o == r) for r in range(2)]
    assert abs(loads[0] - loads[1]) <= 2


def test_balanced_order_at_scale():
    """The c1 list's costs dealt to 8 ranks: vectorised (well under a second for 100k items, and
    for 3.45M), every rank within the largest single cost of every other."""
    import time
    from libcint_gb300 import molecules as M
    from libcint_gb300.dist import quartet_costs
    mol = M.config1(seed=0)
    qs = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'c1_quartets.npz'))['quartets']
    costs = quartet_costs(mol, qs)
    t = time.perf_counter()
    owner = balanced_order(costs, 8)
    assert time.perf_counter() - t < 1.0
    loads = np.bincount(owner, weights=costs, minlength=8)
    assert loads.max() - loads.min() <= costs.max()
    big = np.tile(costs, 35)
    t = time.perf_counter()
    balanced_order(big, 8)
    assert time.perf_counter() - t < 5.0


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
    mgr = mp.get_context('spawn').Manager()
    result = mgr.dict()
    mp.spawn(_worker, args=(2, port, result), nprocs=2, join=True)
    rng = np.random.RandomState(0)
    vals = rng.normal(size=(1000, 5))
    for r in range(2):
        acc, t = result[r]
        np.testing.assert_allclose(acc, vals.sum(0), rtol=1e-12, atol=1e-12)
        assert t == 2.0


def _jk_worker(rank, world, port, result):
    import torch
    import torch.distributed as dist
    from libcint_gb300.dist import shard_quartets, sum_over_ranks
    from tests import _oracle
    from tests.test_jk_algebra import _basis, _contract
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    oracle = _oracle.load()
    mol = _basis()
    mine = shard_quartets(mol, M.unique_quartets(mol.nbas), rank, world)
    blocks = {tuple(int(x) for x in q): oracle.port.call('int2e_sph', mol, q)[1] for q in mine}
    n = mol.ao_loc()[-1]
    d = np.random.RandomState(2).normal(0, 0.3, (n, n))
    J, K = _contract(mol, blocks, 0.5 * (d + d.T), kernel_order=True)
    J, K = torch.tensor(J), torch.tensor(K)
    sum_over_ranks(J)
    sum_over_ranks(K)
    result[rank] = (len(mine), J.numpy(), K.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_jk(oracle):
    import torch.multiprocessing as mp
    from libcint_gb300.dist import quartet_costs, shard_quartets
    from tests.test_jk_algebra import _basis, _eri_full
    mol = _basis()
    qs = M.unique_quartets(mol.nbas)
    # the shards partition the list and balance the estimated cost
    parts = [shard_quartets(mol, qs, r, 2) for r in range(2)]
    assert sorted(map(tuple, np.concatenate(parts).tolist())) == sorted(map(tuple, qs.tolist()))
    loads = [quartet_costs(mol, p).sum() for p in parts]
    assert abs(loads[0] - loads[1]) <= quartet_costs(mol, qs).max()
    port = 31500 + os.getpid() % 2000
    mgr = mp.get_context('spawn').Manager()
    result = mgr.dict()
    mp.spawn(_jk_worker, args=(2, port, result), nprocs=2, join=True)
    eri, _ = _eri_full(oracle, mol)
    n = eri.shape[0]
    d = np.random.RandomState(2).normal(0, 0.3, (n, n))
    dm = 0.5 * (d + d.T)
    Jref = np.einsum('ijkl,kl->ij', eri, dm)
    Kref = np.einsum('ijkl,jl->ik', eri, dm)
    assert result[0][0] + result[1][0] == len(qs)
    for r in range(2):
        _, J, K = result[r]
        assert np.abs(J - Jref).max() <= 1e-12 * np.abs(Jref).max()
        assert np.abs(K - Kref).max() <= 1e-12 * np.abs(Kref).max()

