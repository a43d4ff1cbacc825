"""Several GPUs: independent problems sharded across ranks, no collective on
the data path.

The reference partitions one mesh across MPI ranks and exchanges halo data
every residual (parallel.jl:276-330).  Here the unit of work is a whole
steady solve (a batch or a serving stream), which needs no exchange, so N
ranks (one process per GPU) each solve their own share:

* ``shard`` gives rank r its problems: largest first, each to the rank with the
  least work so far (longest-processing-time order), so the ranks finish
  together;
* the only collectives are on the host side of the measurement: the timed
  region ends with a barrier, the time is the maximum over ranks, and the
  whole-job count is the sum of every rank's units (``job_rate``).
"""
from __future__ import annotations

import heapq


def shard(work, world):
    """Assignment of items (estimated work per item, any non-negative
    numbers) to `world` ranks: a list of index lists, one per rank, each in
    input order.  Deterministic (ties go to the lowest rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return [sorted(x) for x in out]


def my_share(items, work, rank, world):
    """the items of `rank` (see shard)."""
    return [items[i] for i in shard(work, world)[rank]]


def job_rate(units, seconds, dist=None):
    """whole-job rate: the sum of every rank's units over the slowest rank's
    time (dist: an initialised torch.distributed module, or None for one
    rank).  Returns (rate, total units, max seconds)."""
    if dist is None:
        return units / seconds, units, seconds
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    u = torch.tensor([float(units)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t, u = t.cuda(), u.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / float(t.item()), float(u.item()), float(t.item())
