"""Slices across GPUs: one process per GPU, each reconstructing its own
share of an independent-slice workload (a batch of OSEM slices, a volume's
slices), with no collective on the data path.

pyraft reconstructs slice by slice in one process (pyraft/sinogram/sino.py:
284-311 loops over a volume's slices in Python); slices never exchange data,
so the multi-GPU form is a partition of the slice list.  The partition is
by cost (pixels x views per slice, the update count of one EM pass), longest
first onto the least-loaded rank, so ranks finish together even when slice
sizes differ by 64x, and it is deterministic: every rank computes the same
assignment without communicating.  The only collective is the timing
reduction after the work (max over ranks).
"""
from __future__ import annotations

import heapq


def partition(costs, world):
    """Assign slice indices to `world` ranks, longest processing time first.

    Returns a list of `world` sorted index lists, disjoint and covering
    range(len(costs)).  Ties break by index and rank, so the result is the
    same on every rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in out]


def rank_slices(costs, rank, world):
    """This rank's slice indices (see partition)."""
    return partition(costs, world)[rank]


def loads(costs, parts):
    """Total cost per rank of a partition."""
    return [sum(float(costs[i]) for i in p) for p in parts]


def max_over_ranks(value, device=None):
    """Max of a float over the ranks of the default process group (the value
    itself without one).  The only collective of a sharded run."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)
