"""Multi-GPU partitioning of the path (one process per GPU, torch.distributed).

Shell quartets are independent, so a list is split into contiguous rank slices with no exchange
on the data path; J matrices and gradients, which are sums over quartets, need one sum over
ranks at the end; timings take the maximum over ranks.  Works with the nccl and gloo backends
(gloo is what the CPU tests run)."""
import numpy as np


def rank_slice(n, rank, world):
    """[start, end) of rank's contiguous share of n items (sizes differ by at most one)."""
    q, r = divmod(n, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def shard(items, rank, world):
    a, b = rank_slice(len(items), rank, world)
    return items[a:b]


def max_over_ranks(value, device=None):
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(tensor):
    """In-place sum of a J matrix or gradient over ranks."""
    import torch.distributed as dist
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(tensor)
    return tensor


def balanced_order(costs, world):
    """Assignment of items with the given costs to world ranks; returns the rank of every item
    (used when per-item costs vary by orders of magnitude).  Items sorted by cost, longest first,
    are dealt out in rounds of `world`, the direction alternating every round (a serpentine
    deal): vectorised, and any two ranks' loads differ by at most the largest single cost."""
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind='stable')
    k = np.arange(len(costs), dtype=np.int64)
    rnd, pos = k // world, k % world
    owner = np.empty(len(costs), dtype=np.int64)
    owner[order] = np.where(rnd % 2 == 0, pos, world - 1 - pos)
    return owner


def quartet_costs(mol, quartets):
    """Relative cost of each shell quartet: primitive quartets x Cartesian components x
    contraction-column combinations (each combination is its own task)."""
    from .molecules import ANG_OF, NCTR_OF, NPRIM_OF
    q = np.asarray(quartets, dtype=np.int64).reshape(-1, 4)
    l = mol.bas[:, ANG_OF].astype(np.int64)
    per = mol.bas[:, NPRIM_OF].astype(np.float64) * ((l + 1) * (l + 2) // 2) \
        * mol.bas[:, NCTR_OF].astype(np.float64)
    return np.prod(per[q], axis=1)


def shard_quartets(mol, quartets, rank, world):
    """This rank's quartets of a list, balanced by estimated cost (longest processing time)."""
    quartets = np.asarray(quartets)
    if world == 1:
        return quartets
    return quartets[balanced_order(quartet_costs(mol, quartets), world) == rank]


def get_jk_sharded(mol, dm, with_j=True, with_k=True, quartets=None):
    """J and K over all ranks: each rank contracts its cost-balanced share of the unique quartet
    list on its own GPU, then one sum over ranks (the path's only exchange)."""
    import torch.distributed as dist
    from .coulomb import CoulombPlans
    from .molecules import unique_quartets
    rank = dist.get_rank() if dist.is_initialized() else 0
    world = dist.get_world_size() if dist.is_initialized() else 1
    qs = unique_quartets(mol.nbas) if quartets is None else np.asarray(quartets)
    plans = CoulombPlans(mol, shard_quartets(mol, qs, rank, world))
    J, K = plans.get_jk(dm, with_j, with_k)
    for t in (J, K):
        if t is not None:
            sum_over_ranks(t)
    return J, K

