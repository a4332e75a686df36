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
    """Longest-processing-time assignment of items with the given costs to world ranks;
    returns the rank of every item (used when per-item costs vary by orders of magnitude)."""
    order = np.argsort(-np.asarray(costs, dtype=np.float64), kind='stable')
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return owner
