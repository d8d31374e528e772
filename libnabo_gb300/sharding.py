"""Splitting one search over several GPUs (one process per GPU).

Queries are independent, so a search shards without any exchange on the
data path: every rank holds a replica of the cloud's tree (built from the
same host cloud) and searches a contiguous range of the queries; the ranges
are gathered back in rank order, so the result equals the single-GPU one,
and only the TOUCH_STATISTICS counts are summed. Batches of clouds shard by
cloud instead, with a greedy longest-processing-time assignment on the cost
N * Q * k of each cloud.

The functions take a `torch.distributed` process group (NCCL between GPUs,
gloo for CPU tests) or run single-process when `world == 1`.
"""
from __future__ import annotations

import numpy as np


def query_ranges(nq: int, world: int):
    """Contiguous [lo, hi) query ranges, one per rank, sizes differing by at most 1."""
    base, extra = divmod(int(nq), int(world))
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def balance_clouds(costs, world: int):
    """Cloud indices per rank: each cloud, most expensive first, goes to the
    rank with the least total cost so far (ties to the lower rank); returns
    (per-rank index lists in ascending order, per-rank total cost)."""
    costs = np.asarray(costs, dtype=np.float64)
    load = np.zeros(world)
    owner = np.empty(costs.shape[0], dtype=np.int64)
    for c in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        owner[c] = r
        load[r] += costs[c]
    return [np.nonzero(owner == r)[0].tolist() for r in range(world)], load.tolist()


def cloud_costs(point_counts, query_counts, ks):
    """The assignment cost of each cloud of a batch: N * Q * k."""
    return (np.asarray(point_counts, np.float64) * np.asarray(query_counts, np.float64)
            * np.asarray(ks, np.float64))


def search_sharded(search, queries, k: int, rank: int, world: int, group=None):
    """Runs `search(query_block) -> (indices, dists2, touched)` on this rank's
    range of `queries` (the whole array on every rank) and returns the full
    (indices, dists2, touched) on every rank: ranges gathered in rank order,
    touched summed over ranks. `search` works on host numpy arrays."""
    lo, hi = query_ranges(queries.shape[0], world)[rank]
    idx, d2, touched = search(queries[lo:hi])
    if world == 1:
        return idx, d2, int(touched)
    import torch
    import torch.distributed as dist

    sizes = [h - l for l, h in query_ranges(queries.shape[0], world)]
    width = max(sizes)

    def gather(a, fill):
        t = torch.full((width, k), fill, dtype=torch.from_numpy(a[:0]).dtype)
        t[: a.shape[0]] = torch.from_numpy(np.ascontiguousarray(a))
        parts = [torch.empty_like(t) for _ in range(world)]
        dist.all_gather(parts, t, group=group)
        return np.concatenate([p[:n].numpy() for p, n in zip(parts, sizes)])

    all_idx = gather(np.asarray(idx), -1)
    all_d2 = gather(np.asarray(d2), 0)
    t = torch.tensor([int(touched)], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return all_idx, all_d2, int(t.item())


def batch_sharded(search_clouds, point_counts, query_counts, ks, rank: int, world: int, group=None):
    """Batches: this rank searches its clouds (`search_clouds(list of cloud
    indices) -> {cloud: (indices, dists2)}`); the per-cloud results of all
    ranks are gathered into one dict on every rank."""
    mine, _ = balance_clouds(cloud_costs(point_counts, query_counts, ks), world)
    res = search_clouds(mine[rank])
    if world == 1:
        return res
    import torch.distributed as dist

    everything = [None] * world
    dist.all_gather_object(everything, res, group=group)
    out = {}
    for part in everything:
        out.update(part)
    return out
