"""Independent systems shared out over the ranks of a job, one process per GPU.

The path has no exchange step: every solve (one lattice, one source of a multishift solve,
one system of a batch) is independent.  A job with several GPUs therefore gives each rank a
share of the systems, solves its share with no collective on the data path, and only gathers
the small per-system results (iteration counts, residuals) and the timing at the end.  The
reference solves one system per call and has no multi-process layer; this module is the
host-side logic of the multi-GPU mode, and runs unchanged on CPU ranks (gloo) in the tests.
"""
from __future__ import annotations

import heapq


def shard_by_cost(costs, world):
    """Split systems 0..len(costs)-1 over `world` ranks, balancing the summed cost (for example,
    sites x expected iterations): largest first, each to the least-loaded rank (ties to the
    lower rank).  Returns one ascending index list per rank; every index appears once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    shares = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def my_share(costs, rank, world):
    """This rank's systems (shard_by_cost)."""
    return shard_by_cost(costs, world)[rank]


def gather_results(local, world):
    """Every rank passes {system index: result}; returns the union on every rank (small host
    objects only, through torch.distributed.all_gather_object).  world == 1 returns `local`."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, dict(local))
    out = {}
    for p in parts:
        overlap = out.keys() & p.keys()
        if overlap:
            raise RuntimeError(f"systems solved on two ranks: {sorted(overlap)}")
        out.update(p)
    return out


def max_over_ranks(value, world, device=None):
    """The largest `value` over the ranks (a job's time is its slowest rank's)."""
    if world == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
