"""Autotuner for batched searches.

Times the batched build + search (one CUDA-graph launch) on a sample of the
batch for every candidate configuration -- kd-tree bucket size, split rule
(the reference's sliding midpoint, or the median: a balanced tree with the
same layout), threads per query (one thread, or a group of 8 lanes sharing
one traversal with the top-k spread over their registers) and threads per
block of the search kernel -- and keeps the fastest. Every configuration returns the exact neighbours; only speed
differs. The median split builds another tree than the reference's, so
callers that need the reference's own trees pass ``split_rules=(0,)``. Choices are cached per workload shape (dimension, scalar
type, largest k, point-count scale), in memory and optionally in a JSON file.
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

CANDIDATES = {"bucketSize": (4, 6, 8, 12, 16, 24, 32), "threadsPerBlock": (64, 128), "splitRule": (0, 1),
              "lanesPerQuery": (1, 8)}
_cache: dict = {}


def shape_key(point_counts, dim, dtype, k) -> str:
    mean = float(np.mean(point_counts))
    return f"d{dim}-{np.dtype(dtype).name}-k{int(np.max(k))}-n2^{int(round(math.log2(max(mean, 1.0))))}"


def _time_config(clouds, queries, pc, qc, ks, dim, dtype, bucket, tpb, rule, lanes, repeats):
    import torch

    from . import BatchSearch
    b = BatchSearch(pc, dim=dim, dtype=dtype, bucketSize=bucket, threadsPerBlock=tpb, splitRule=rule,
                    lanesPerQuery=lanes)
    b.set_queries(qc, ks)
    out = b._outputs(queries.device)
    b.run(clouds, queries, out=out)  # capture + first launch
    torch.cuda.synchronize()
    st = b.status()
    if not st["ok"]:
        b.close()
        return math.inf, st
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = math.inf
    for _ in range(repeats):
        ev0.record()
        b.run(clouds, queries, out=out)
        ev1.record()
        torch.cuda.synchronize()
        best = min(best, ev0.elapsed_time(ev1))
    b.close()
    return best, st


def _levels_of(cloud, queries, k, dim, dtype, bucket, rule) -> int:
    """Top-phase levels the forest build needs for one cloud."""
    import torch

    from . import BatchSearch
    b = BatchSearch([cloud.shape[0]], dim=dim, dtype=dtype, bucketSize=bucket, maxLevels=256, splitRule=rule)
    b.set_queries([0], [k])
    b.build(torch.from_numpy(np.ascontiguousarray(cloud, dtype=dtype)).cuda())
    torch.cuda.synchronize()
    levels = b.status()["levels"]
    b.close()
    return int(levels)


def tune(cloud_list, query_list, k, dim: int = 3, dtype=np.float32, sample: int = 64, repeats: int = 3,
         cache_path: str | None = None, seed: int = 0, split_rules=CANDIDATES["splitRule"],
         max_queries_per_cloud: int | None = None, lanes=None) -> dict:
    """Best {bucketSize, threadsPerBlock, splitRule, lanesPerQuery} for a batch (lists of (n_c, dim)
    arrays), timed on `sample` of its clouds with at most `max_queries_per_cloud` of each one's
    queries; `lanes` restricts the lanes-per-query candidates."""
    import torch
    ks = np.broadcast_to(np.asarray(k, dtype=np.int32), (len(cloud_list),))
    pcs = np.array([c.shape[0] for c in cloud_list], np.int64)
    split_rules = tuple(int(r) for r in split_rules)
    lane_set = tuple(int(x) for x in (lanes if lanes is not None else CANDIDATES["lanesPerQuery"]))
    key = shape_key(pcs, dim, dtype, ks) + ("" if split_rules == (0, 1) else "-s" + "".join(map(str, split_rules)))
    key += "" if lane_set == CANDIDATES["lanesPerQuery"] else "-l" + "".join(map(str, lane_set))
    if key in _cache:
        return dict(_cache[key], key=key, cached=True)
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            disk = json.load(f)
        if key in disk:
            _cache[key] = disk[key]
            return dict(disk[key], key=key, cached=True)
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(len(cloud_list), min(sample, len(cloud_list)), replace=False))
    pc = pcs[pick]
    qsub = [query_list[i][:max_queries_per_cloud] if max_queries_per_cloud else query_list[i] for i in pick]
    qc = np.array([q.shape[0] for q in qsub], np.int64)
    clouds = torch.from_numpy(np.concatenate([cloud_list[i] for i in pick]).astype(dtype)).cuda()
    queries = torch.from_numpy(np.concatenate(qsub).astype(dtype)).cuda()
    trials = []
    t0 = time.perf_counter()
    # lane groups apply to k <= 32 and run blocks of 128 threads
    lane_choices = lane_set if int(np.max(ks)) <= 32 else (1,)
    for rule in split_rules:
        for bucket in CANDIDATES["bucketSize"]:
            for lanes in lane_choices:
                for tpb in (CANDIDATES["threadsPerBlock"] if lanes == 1 else (128,)):
                    ms, st = _time_config(clouds, queries, pc, qc, ks[pick], dim, dtype, bucket, tpb, rule, lanes,
                                          repeats)
                    trials.append({"bucketSize": bucket, "threadsPerBlock": tpb, "splitRule": rule,
                                   "lanesPerQuery": lanes, "ms": ms, "levels": st["levels"]})
    best = min(trials, key=lambda t: t["ms"])
    # the fixed level count must cover the batch's largest cloud, sampled or not
    levels = best["levels"]
    big = int(np.argmax(pcs))
    if big not in set(pick.tolist()):
        levels = max(levels, _levels_of(cloud_list[big], query_list[big], int(ks[big]), dim, dtype,
                                        best["bucketSize"], best["splitRule"]))
    choice = {"bucketSize": best["bucketSize"], "threadsPerBlock": best["threadsPerBlock"],
              "splitRule": best["splitRule"], "lanesPerQuery": best["lanesPerQuery"],
              "maxLevels": max(8, levels + 8), "sample_ms": best["ms"]}
    _cache[key] = choice
    if cache_path:
        disk = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                disk = json.load(f)
        disk[key] = choice
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(disk, f, indent=1)
    return dict(choice, key=key, cached=False, trials=trials, tune_s=time.perf_counter() - t0)
