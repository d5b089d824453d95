"""Batches over several GPUs: one process per GPU, pairs partitioned across
the processes, results gathered on the host.

Pairs are independent, so a batch shards with no exchange on the data path:
every rank runs its own share through its own context (one persistent launch
per rank) and the ranks swap only their result records afterwards (a
host-side gather, any ``torch.distributed`` backend, gloo included).

The reference has no multi-GPU path (its device is a compile-time constant,
forBench/HausdorffDistance.cuh:5); this module is the batching layer's
scale-out.  The split is greedy largest-first (longest-processing-time) on a
per-pair cost.  The cost that is known before the run is the volume W*H*D:
the work of a pair is its voxel-iterations, and the iteration count (the
distance) is only known afterwards.
"""
from __future__ import annotations

import heapq
from typing import Callable, Optional, Sequence


def pair_cost(a) -> int:
    """Cost proxy of one pair: its voxel count (shape (D, H, W))."""
    s = tuple(int(x) for x in a.shape)
    n = 1
    for x in s:
        n *= x
    return n


def plan_shards(costs: Sequence[float], world_size: int) -> list:
    """Greedy largest-first split of pairs over ranks.

    Returns one list of pair indices per rank (each list ascending).  Pairs
    are taken in decreasing cost (ties by index) and each goes to the rank
    with the least total so far (ties by rank), so the largest load is at
    most 4/3 of the optimum.  Deterministic: every rank computes the same plan.
    """
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world_size)]
    shards = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shards]


def batch_sharded(pairs: Sequence, compute: Callable[[list], list], *, costs: Optional[Sequence[float]] = None,
                  group=None) -> list:
    """Run a batch split across the ranks of a process group.

    ``compute(list_of_pairs) -> list_of_results`` runs one rank's share (for a
    GPU rank: ``ctx.batch`` with a bound metric).  Every rank passes the same
    ``pairs`` list (shapes only are used for planning) and gets back every
    pair's result in input order.  Without an initialised process group the
    whole batch runs locally.
    """
    import torch.distributed as dist

    if group is None and not (dist.is_available() and dist.is_initialized()):
        return list(compute(list(pairs)))
    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    if costs is None:
        costs = [pair_cost(p[0]) for p in pairs]
    if len(costs) != len(pairs):
        raise ValueError("one cost per pair")
    shards = plan_shards(costs, ws)
    mine = shards[rank]
    res = list(compute([pairs[i] for i in mine])) if mine else []
    if len(res) != len(mine):
        raise RuntimeError(f"rank {rank}: compute returned {len(res)} results for {len(mine)} pairs")
    gathered = [None] * ws
    dist.all_gather_object(gathered, list(zip(mine, res)), group=group)
    out = [None] * len(pairs)
    for part in gathered:
        for i, r in part:
            out[i] = r
    missing = [i for i, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError(f"pairs without a result after the gather: {missing[:8]}")
    return out
