"""Replica sharding across ranks (one process per GPU).

Restarts, cells and requests are independent instances, so N GPUs run N
disjoint instance sets with no data-path collective; the only exchange is
the timing summary at the end: the slowest rank's time and the units of all
ranks.
"""
from .workloads import instance_seed


def rank_seeds(base, rank, count):
    """Seeds of `count` instances owned by `rank`: rank r uses the
    covengine-style stream of base + 7919 r, so no two ranks share one."""
    return [instance_seed(base + 7919 * rank, i) for i in range(count)]


def shard(items, rank, world):
    """Round-robin share of a global instance list for one rank."""
    return items[rank::world]


def combine(dist, ms, units, device=None):
    """(max ms over ranks, sum of units over ranks); identity without dist."""
    if dist is None:
        return float(ms), float(units)
    import torch
    t_max = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    t_sum = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    dist.all_reduce(t_sum, op=dist.ReduceOp.SUM)
    return float(t_max[0]), float(t_sum[0])
