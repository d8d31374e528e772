#!/usr/bin/env python
"""Throughput benchmark of the GB300 kNN path; prints one JSON line.

Workload (default ``lidar``): the synthetic 64-beam lidar scan (about 1.15 M
float32 points, 3-D), queried by the same scan after a random 2-degree
rotation and a 0.1 m translation; k = 10, maxRadius = 1.0 m, self-match off,
bucketSize 8 -- exact kNN through the CUDA kd-tree. ``--workload uniform``
runs 1 M uniform points against 1 M uniform queries, k = 10.

One step = one kNN search of every query of the batch.
  value  queries/s with the cloud's tree and the queries already in HBM
         (device API, CUDA events around each step, L2 flushed between steps)
  e2e    the same search through the host API (nabo_cuda_knn) from pinned
         host buffers: query upload, search, result download, per step
  roofline  algorithmic bytes of the search kernel / its event-timed duration
  cpu_baseline  the oracle's restatement of the reference's OpenMP
         KDTREE_LINEAR_HEAP search timed on this host's cores

``--impl reference`` times the reference algorithm on the host CPU instead
(the C++ restatement in oracle/, all host threads) on the same workload.
Multi-GPU (torchrun): every rank builds a replica of the tree and searches
its own query batch (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "exact kNN queries/s (1M-pt 3D, k=10): learned-radius vs plain GPU kd-tree"
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["lidar", "uniform", "c0", "batched", "c4", "bf", "latency"], default="lidar",
                   help="batched: 512 uneven 3-D clouds built and searched per step (one CUDA graph); "
                        "c4: 128 8-D clouds (half f32, half f64), k=32, epsilon 0 and 0.5")
    p.add_argument("--c4-clouds", type=int, default=128, help="clouds of the c4 workload (a prefix of the 128)")
    p.add_argument("--k", type=int, default=10)
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-order", action="store_true", help="keep the queries in their given order")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-radius form")
    p.add_argument("--train-queries", type=int, default=200000)
    p.add_argument("--split-rules", default="0,1",
                   help="batched workload: split rules the autotuner may choose (0 the reference's, 1 median)")
    p.add_argument("--traversal", type=int, default=0,
                   help="kd-tree traversal: 0/1 reference visit order (default), 2 warp packet")
    return p.parse_args()


def workload(name: str, rank: int):
    from libnabo_gb300 import synthetic as S
    if name == "lidar":
        cloud = S.lidar_scan()
        q = S.lidar_queries(cloud, seed=S.SEED_BASE + 1 + 7919 * rank)
        return cloud, q, dict(maxRadius=1.0, flags=0, label="lidar64_1.15M")
    if name == "c0":  # the reference's small CPU-runnable case: 10,000 uniform points and queries
        cloud = S.uniform(10_000, 3, seed=S.SEED_BASE + 7)
        q = S.uniform(10_000, 3, seed=S.SEED_BASE + 8 + 7919 * rank)
        return cloud, q, dict(maxRadius=float("inf"), flags=0, label="uniform_10k")
    cloud = S.uniform(1_000_000, 3, seed=S.SEED_BASE + 5)
    q = S.uniform(1_000_000, 3, seed=S.SEED_BASE + 6 + 7919 * rank)
    return cloud, q, dict(maxRadius=float("inf"), flags=0, label="uniform_1M")


def training_queries(name: str, q, count: int):
    """Training queries for the radius network, disjoint from the timed ones.
    Lidar: another frame -- the same scene scanned again with fresh range
    noise, moved by the same pose change as the timed queries (a query's k-th
    distance is dominated by how far that motion moved it off the surfaces),
    as frame t trains the network a sensor loop uses on frame t + 1; uniform:
    fresh samples of the same law."""
    from libnabo_gb300 import synthetic as S
    rng = np.random.default_rng(S.SEED_BASE + 4242)
    if name == "lidar":
        frame = S.lidar_queries(S.lidar_scan(noise_seed=S.SEED_BASE + 4244))
        return frame[rng.choice(frame.shape[0], min(count, frame.shape[0]), replace=False)]
    return S.uniform(count, 3, seed=S.SEED_BASE + 4243)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(label: str, k: int):
    """DRAM bytes per launch of the search kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"knn_kdtree_{label}_k{k}.txt")
    if not os.path.exists(path):
        return None, None
    per_launch, nq = None, None
    with open(path) as f:
        for line in f:
            if line.startswith("dram_bytes_per_launch:"):
                per_launch = float(line.split(":", 1)[1])
            if line.startswith("queries_per_launch:"):
                nq = float(line.split(":", 1)[1])
    return per_launch, nq


def _nvtx_timed(push: bool) -> None:
    """An NVTX range named "timed" around the timed steps, so that a profiler
    can capture just their kernels (ncu --nvtx --nvtx-include "timed/")."""
    try:
        import torch
        if push:
            torch.cuda.nvtx.range_push("timed")
        else:
            torch.cuda.nvtx.range_pop()
    except (ImportError, RuntimeError, AttributeError):
        pass


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms, over the
    timed steps (which it also marks with the "timed" NVTX range)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = f"/tmp/nabo_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        _nvtx_timed(True)
        return self

    def __exit__(self, *exc):
        _nvtx_timed(False)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(cloud, q, k, cfg, reps=5):
    """The reference's OpenMP KDTREE_LINEAR_HEAP search (oracle restatement)
    on all host threads: build time and best-of-`reps` query throughput."""
    from oracle import oracle as O
    threads = O.num_threads()
    t0 = time.perf_counter()
    tree = O.OracleTree(cloud, bucket_size=8)
    build_s = time.perf_counter() - t0
    tree.knn(q[:10000], k, 0.0, cfg["flags"], cfg["maxRadius"], mode=O.MODE_REFERENCE)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        tree.knn(q, k, 0.0, cfg["flags"], cfg["maxRadius"], mode=O.MODE_REFERENCE)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    stats_tree = O.OracleTree(cloud, bucket_size=8, creation_flags=O.TOUCH_STATISTICS)
    sample = q
    _, _, touched = stats_tree.knn(sample, k, 0.0, cfg["flags"], cfg["maxRadius"], mode=O.MODE_REFERENCE)
    return {"value": q.shape[0] / best, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"all {q.shape[0]} queries of the workload, best of {reps} after 1 warm-up; "
                      f"tree build {build_s:.3f} s single-threaded",
            "build_s": build_s, "touched_per_query": touched / sample.shape[0]}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    cloud, q, cfg = workload(args.workload, 0)
    k = args.k
    tree = O.OracleTree(cloud, bucket_size=8)
    for _ in range(max(args.warmup, 1)):
        tree.knn(q, k, 0.0, cfg["flags"], cfg["maxRadius"], mode=O.MODE_REFERENCE)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tree.knn(q, k, 0.0, cfg["flags"], cfg["maxRadius"], mode=O.MODE_REFERENCE)
        times.append(time.perf_counter() - t0)
    per = sum(times) / len(times)
    value = q.shape[0] / per
    threads = O.num_threads()
    out = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": f"{cfg['label']}_k{k}", "points": int(cloud.shape[0]), "queries": int(q.shape[0]),
                   "k": k, "maxRadius": cfg["maxRadius"], "bucketSize": 8,
                   "search": "KDTREE_LINEAR_HEAP restated in C++/OpenMP (oracle/nabo_oracle.cpp)"},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"all {q.shape[0]} queries per step"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_ours(args):
    import torch
    import torch.distributed as dist

    import libnabo_gb300 as nb

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    k = args.k
    cloud, q, cfg = workload(args.workload, rank)
    nq = q.shape[0]
    stream = torch.cuda.current_stream(dev)

    # build (timed separately, reported as a side figure)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    params = {"bucketSize": 8, "traversal": args.traversal, "queryOrdering": 0 if args.no_order else 1}
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params=params)
    build_s = time.perf_counter() - t0
    # a second build after warm-up is the steady-state figure
    s.close()
    t0 = time.perf_counter()
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params=params)
    build_s = min(build_s, time.perf_counter() - t0)
    s_stats = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)

    tq = torch.from_numpy(q).to(dev)
    idx = torch.empty((nq, k), dtype=torch.int32, device=dev)
    d2 = torch.empty((nq, k), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    touched = torch.zeros(1, dtype=torch.int64, device=dev)
    s_stats.knn_device(tq, k, 0.0, cfg["flags"], cfg["maxRadius"], out=(idx, d2), touched=touched)
    torch.cuda.synchronize()
    p_bar = int(touched.item()) / nq
    s.profile(True)

    def timed(step_fn, kernel_ms_fn=None):
        """W warm-up steps, then K steps timed with CUDA events (L2 flushed
        before each); returns (per-step ms list, kernel ms list)."""
        for _ in range(args.warmup):
            flush.zero_()
            step_fn()
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kms = []
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step_fn()
            ends[i].record(stream)
            if kernel_ms_fn is not None:
                kms.append(kernel_ms_fn())
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return [a.elapsed_time(b) for a, b in zip(starts, ends)], kms

    def max_over_ranks(x):
        if world > 1:
            t = torch.tensor([x], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    def plain_step():
        s.knn_device(tq, k, 0.0, cfg["flags"], cfg["maxRadius"], out=(idx, d2))

    with ClockSampler(local) as clk:
        step_ms, kernel_ms = timed(plain_step, s.last_kernel_ms)
        plain_ms = max_over_ranks(sum(step_ms)) / args.steps
        learned = None
        if not args.no_learned:
            tr = training_queries(args.workload, q, args.train_queries)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            model = nb.RadiusModel(s, tr, k=k, optionFlags=cfg["flags"], maxRadius=cfg["maxRadius"])
            torch.cuda.synchronize()
            train_s = time.perf_counter() - t0
            fb = torch.zeros(1, dtype=torch.int32, device=dev)
            li = torch.empty_like(idx)
            ld = torch.empty_like(d2)

            def learned_step():
                model.knn_device(tq, k, 0.0, cfg["flags"], cfg["maxRadius"], out=(li, ld), fallbacks=fb)

            lstep_ms, lkernel_ms = timed(learned_step, s.last_kernel_ms)
            learned_ms = max_over_ranks(sum(lstep_ms)) / args.steps
            torch.cuda.synchronize()
            exact = bool(torch.equal(li, idx) and torch.equal(ld, d2))
            # the best any radius predictor can do: each query's exact k-th
            # distance (a hair above it) as its radius, no misses
            ideal = torch.where(idx[:, -1] >= 0, torch.sqrt(d2[:, -1]) * (1.0 + 2.0 ** -20),
                                torch.full_like(d2[:, -1], cfg["maxRadius"])).contiguous()
            ii = torch.empty_like(idx)
            idd = torch.empty_like(d2)

            def ideal_step():
                s.knn_device(tq, k, 0.0, cfg["flags"], cfg["maxRadius"], maxRadii=ideal, out=(ii, idd))

            _, ideal_kernel_ms = timed(ideal_step, s.last_kernel_ms)
            torch.cuda.synchronize()
            ideal_exact = bool(torch.equal(ii, idx) and torch.equal(idd, d2))
            learned = {"ms_per_step": learned_ms, "queries_per_s": world * nq / (learned_ms / 1e3),
                       "fallbacks": int(fb.item()), "fallback_rate": int(fb.item()) / nq,
                       "identical_to_plain": exact, "train_s": train_s, "train_queries": int(tr.shape[0]),
                       "train_queries_from": "another frame of the scene (fresh range noise, same pose change), disjoint from the timed queries" if args.workload == "lidar"
                       else "independent samples of the query distribution",
                       "bounded_kernel_ms": statistics.mean(lkernel_ms),
                       "ideal_radius_kernel_ms": statistics.mean(ideal_kernel_ms),
                       "ideal_radius_identical": ideal_exact,
                       "model": {kk: (round(v, 6) if isinstance(v, float) else v) for kk, v in model.meta.items()}}
    plain_value = world * nq / (plain_ms / 1e3)
    plain_kernel_ms = statistics.mean(kernel_ms)
    use_learned = learned is not None and learned["identical_to_plain"] and learned["ms_per_step"] < plain_ms
    ms_per_step = learned["ms_per_step"] if use_learned else plain_ms
    value = world * nq / (ms_per_step / 1e3)

    # end to end through the host API, pinned host buffers
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    hq = torch.from_numpy(q).pin_memory().numpy()
    hidx = torch.empty((nq, k), dtype=torch.int32).pin_memory().numpy()
    hd2 = torch.empty((nq, k), dtype=torch.float32).pin_memory().numpy()
    search_api = model if use_learned else s
    for _ in range(2):
        search_api.knn(hq, k, 0.0, cfg["flags"], cfg["maxRadius"], out=(hidx, hd2))
    e2e_t = []
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        search_api.knn(hq, k, 0.0, cfg["flags"], cfg["maxRadius"], out=(hidx, hd2))
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(sum(e2e_t) / len(e2e_t))
    e2e_value = world * nq / e2e_s

    # roofline of the search kernel: algorithmic bytes per query
    #   B_q = D*s + k*(4+s) + P*(D*s + 4)   (query, results, touched points)
    # with P the reference algorithm's touched points (TOUCH_STATISTICS of
    # the unbounded search on the same input)
    dsz, D = 4, 3
    b_q = D * dsz + k * (4 + dsz) + p_bar * (D * dsz + 4)
    kern_s = statistics.mean(lkernel_ms if use_learned else kernel_ms) / 1e3
    achieved = nq * b_q / kern_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic_launch, traffic_nq = profiled_traffic(cfg["label"], k)
    traffic = None
    if traffic_launch is not None and traffic_nq:
        traffic = traffic_launch * nq / traffic_nq

    if rank != 0:
        return
    base = None
    if not args.no_cpu_baseline:
        base = cpu_baseline(cloud, q, k, cfg)
    clocks = clk.summary()
    # the library sorts the queries when the work outweighs the sort (its
    # worth_sorting rule, csrc/internal.cuh). A 3-D sort is Morton keys with
    # the first digit counts, then three 10-bit radix passes (digit scan +
    # scatter each, counts for the last two); then the search kernel.
    sorts = not args.no_order and nq * (k + 10) / 20 * (8 if cloud.shape[1] > 3 else 1) >= 2 ** 18
    launches_per_step = 10 if sorts else 1
    if use_learned:
        launches_per_step += 1  # radius network (misses rerun inside the search kernel)
    out = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{cfg['label']}_k{k}", "points": int(cloud.shape[0]), "queries": int(nq),
                   "k": k, "maxRadius": cfg["maxRadius"], "selfMatch": False, "bucketSize": 8,
                   "form": "learned radius (MLP) + kd-tree" if use_learned else "plain GPU kd-tree",
                   "traversal": "warp packet" if args.traversal == 2 else "reference order",
                   "query_order": "given" if args.no_order else "30-bit Morton code, stable radix sort",
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                "d2h_bytes_per_step": int(hidx.nbytes + hd2.nbytes + 8)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "k_knn_kdtree (bounded search of the learned form)" if use_learned
                     else "k_knn_kdtree", "kernel_ms": kern_s * 1e3, "bytes_per_query": b_q,
                     "touched_per_query": p_bar},
        "forms": {"plain": {"ms_per_step": plain_ms, "queries_per_s": plain_value, "kernel_ms": plain_kernel_ms},
                  "learned": learned},
        "cpu_baseline": base,
        "clocks": clocks,
        "gpu_launches": launches_per_step * args.steps,
        "build_ms": build_s * 1e3,
    }
    if base is not None:
        out["cpu_baseline"] = {kk: base[kk] for kk in ("value", "unit", "cores", "kind", "sample")}
        out["cpu_baseline"]["build_s"] = base["build_s"]
        out["cpu_baseline"]["touched_per_query"] = base["touched_per_query"]
    print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Batched workload: 512 independent 3-D float32 clouds, sizes log-uniform in
# [2,000; 200,000], each a mixture of 8 anisotropic Gaussian blobs (sigma
# 0.05-2.0); each cloud is queried by a copy of itself with per-point noise
# sigma 0.01; k per cloud from {1, 5, 16}. One step = every tree built and
# every query searched, as one CUDA-graph launch (forest build + one search
# kernel), with bucket size and threads per block from the autotuner.

BATCH_METRIC = "batched kNN queries/s (512 uneven 3-D clouds, build + search per step)"


def batched_workload(rank: int, n_clouds: int = 512):
    from libnabo_gb300 import synthetic as S
    seed = S.SEED_BASE + 300 + 7919 * rank
    sizes = S.log_uniform_sizes(n_clouds, 2000, 200000, seed)
    rng = np.random.default_rng(seed + 1)
    clouds = [S.gaussian_blobs(int(n), seed + 10 + i) for i, n in enumerate(sizes)]
    queries = [(c + rng.normal(0, 0.01, c.shape)).astype(np.float32) for c in clouds]
    ks = rng.choice([1, 5, 16], n_clouds).astype(np.int32)
    return clouds, queries, ks


def batched_cpu(clouds, queries, ks, sample: int = 16, seed: int = 0):
    """Oracle (the reference's OpenMP KDTREE_LINEAR_HEAP restated) on a
    sample of the clouds: build + search time, queries/s, touched/query."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(len(clouds), min(sample, len(clouds)), replace=False))
    nq, t_build, t_search, touched = 0, 0.0, 0.0, 0
    for c in pick:
        t0 = time.perf_counter()
        tree = O.OracleTree(clouds[c], bucket_size=8, creation_flags=O.TOUCH_STATISTICS)
        t_build += time.perf_counter() - t0
        t0 = time.perf_counter()
        _, _, tc = tree.knn(queries[c], int(ks[c]), mode=O.MODE_REFERENCE)
        t_search += time.perf_counter() - t0
        nq += queries[c].shape[0]
        touched += int(tc)
    return {"value": nq / (t_build + t_search), "unit": "queries/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{len(pick)} of {len(clouds)} clouds ({nq} queries), tree build + search each",
            "search_only_queries_per_s": nq / t_search, "touched_per_query": touched / nq, "clouds": pick.tolist()}


def run_batched(args):
    import torch
    import torch.distributed as dist

    import libnabo_gb300 as nb
    from libnabo_gb300 import autotune

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    clouds, queries, ks = batched_workload(rank)
    pc = np.array([c.shape[0] for c in clouds], np.int64)
    qc = np.array([q.shape[0] for q in queries], np.int64)
    t0 = time.perf_counter()
    choice = autotune.tune(clouds, queries, ks, sample=64, repeats=3,
                           split_rules=tuple(int(r) for r in args.split_rules.split(",")))
    tune_s = time.perf_counter() - t0
    b = nb.BatchSearch(pc, bucketSize=choice["bucketSize"], threadsPerBlock=choice["threadsPerBlock"],
                       maxLevels=choice["maxLevels"], splitRule=choice["splitRule"],
                       lanesPerQuery=choice.get("lanesPerQuery", 1))
    b.set_queries(qc, ks)
    hc = np.concatenate(clouds)
    hq = np.concatenate(queries)
    tc = torch.from_numpy(hc).to(dev)
    tq = torch.from_numpy(hq).to(dev)
    out = b._outputs(dev)
    nq_total = int(qc.sum())

    def step():
        b.run(tc, tq, out=out)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    st = b.status()
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for e0, e1 in ev:
            e0.record()
            step()
            e1.record()
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms = max_ranks(sum(e0.elapsed_time(e1) for e0, e1 in ev) / args.steps, world)
    # phases outside the graph (same kernels): forest build, then search
    b.build(tc)
    torch.cuda.synchronize()
    tb = []
    ts = []
    for _ in range(3):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        b.build(tc)
        e1.record()
        b.knn(tq, out=out)
        e2.record()
        torch.cuda.synchronize()
        tb.append(e0.elapsed_time(e1))
        ts.append(e1.elapsed_time(e2))
    build_ms, search_ms = min(tb), min(ts)
    # exactness on a few clouds against the oracle
    from oracle import oracle as O
    gi = b.split(out[0].cpu().numpy())
    gd = b.split(out[1].cpu().numpy())
    checked, same = 0, True
    for c in range(0, len(clouds), max(1, len(clouds) // 8)):
        # the exact k smallest pairs (the reference's tree or the median-split
        # one, whichever the autotuner chose, returns them)
        oi, od, _ = O.bf_knn(clouds[c], queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        same = same and np.array_equal(gi[c], oi) and np.array_equal(gd[c].view(np.uint32), od.view(np.uint32))
        checked += 1
    # end to end through the host-buffer call: clouds and queries from pinned
    # host memory, results into pinned host arrays, copies inside the call
    pin_c = torch.from_numpy(hc).pin_memory()
    pin_q = torch.from_numpy(hq).pin_memory()
    h_idx = torch.empty(out[0].shape, dtype=out[0].dtype).pin_memory()
    h_d2 = torch.empty(out[1].shape, dtype=out[1].dtype).pin_memory()
    host_in = (pin_c.numpy(), pin_q.numpy())
    host_out = (h_idx.numpy(), h_d2.numpy())
    b.run_host(*host_in, out=host_out)  # first call captures its graph
    e2e_same = bool(np.array_equal(host_out[0], out[0].cpu().numpy())
                    and np.array_equal(host_out[1].view(np.uint32), out[1].cpu().numpy().view(np.uint32)))
    e2e_steps = args.e2e_steps or max(10, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        b.run_host(*host_in, out=host_out)
    e2e_s = max_ranks((time.perf_counter() - t0) / e2e_steps, world)
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    base = None if args.no_cpu_baseline else batched_cpu(clouds, queries, ks)
    peak, peak_kind = measured_peaks()
    p_bar = base["touched_per_query"] if base else None
    achieved, b_q = None, None
    if p_bar is not None:
        s = 4
        mean_k = float(np.sum(qc * ks) / nq_total)
        b_q = 3 * s + mean_k * (4 + s) + p_bar * (3 * s + 4)
        achieved = nq_total * b_q / (search_ms * 1e-3) / 1e9
    res = {
        "metric": BATCH_METRIC, "value": world * nq_total / (step_ms / 1e3), "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched512_3d", "clouds": len(clouds), "points": int(pc.sum()),
                   "queries": nq_total, "k": "per cloud from {1, 5, 16}", "selfMatch": False,
                   "bucketSize": choice["bucketSize"], "threadsPerBlock": choice["threadsPerBlock"],
                   "splitRule": choice["splitRule"], "lanesPerQuery": choice.get("lanesPerQuery", 1),
                   "maxLevels": choice["maxLevels"], "autotune_s": tune_s,
                   "autotune_trials": choice.get("trials"),
                   "step": "forest build + search, one CUDA graph launch",
                   "l2": "inputs larger than L2 (clouds + queries %.0f MB)" % ((hc.nbytes + hq.nbytes) / 1e6),
                   "parallelism": f"replicas x{world}"},
        "phases_ms": {"build": build_ms, "search": search_ms},
        "status": st, "exact_vs_oracle": {"clouds_checked": checked, "identical": bool(same)},
        "e2e": {"value": world * nq_total / e2e_s, "unit": "queries/s", "call": "BatchSearch.run_host",
                "equals_device_run": e2e_same,
                "h2d_bytes_per_step": int(hc.nbytes + hq.nbytes),
                "d2h_bytes_per_step": int(h_idx.numel() * 4 + h_d2.numel() * 4)},
        "roofline": None if achieved is None else {
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_kind,
            "kernel": "batched search call (query ordering + k_knn_kdtree), event-timed",
            "kernel_ms": search_ms, "bytes_per_query": b_q, "touched_per_query": p_bar},
        "cpu_baseline": None if base is None else {kk: base[kk] for kk in ("value", "unit", "cores", "kind",
                                                                           "sample", "search_only_queries_per_s")},
        "clocks": clk.summary(),
        # per graph launch: forest set-up 6 + 17 per level + small/status/
        # renumber/copy 4; search: leaf cells, 3 scan kernels, placement,
        # run sort, search 7
        "gpu_launches": args.steps * (6 + 17 * choice["maxLevels"] + 4 + 7),
    }
    print(json.dumps(res))
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# 8-D workload: 128 clouds, sizes log-uniform in [50,000; 2,000,000], half
# float32 and half float64, each a mixture of 32 isotropic Gaussian clusters
# with sigma log-uniform in [0.01, 1]; 100,000 queries per cloud from the
# same mixture; k = 32; epsilon 0 (exact) and 0.5 (approximate, within the
# reference's (1+eps) bound). One BatchSearch per scalar type; trees built
# once, a step searches every query of both batches.

C4_METRIC = "batched 8-D kNN queries/s (128 clouds, half f32 / half f64, k=32)"


def c4_workload(n_clouds: int = 128, train_per_cloud: int = 3125):
    """The 8-D batches: clouds, the timed queries (100,000 per cloud) and,
    for the learned form, training queries drawn separately from the same
    mixture (3,125 per cloud: 200,000 per scalar type)."""
    from libnabo_gb300 import synthetic as S
    seed = S.SEED_BASE + 400
    sizes = S.log_uniform_sizes(128, 50000, 2000000, seed)[:n_clouds]
    out = {np.float32: ([], [], []), np.float64: ([], [], [])}
    for i, n in enumerate(sizes):
        dt = np.float32 if i % 2 == 0 else np.float64
        cloud, centres, sig = S.clusters(int(n), 8, seed + 10 + i, dtype=dt)
        qs, _, _ = S.clusters(100000, 8, seed + 10000 + i, dtype=dt, centres=centres, sigmas=sig)
        tr, _, _ = S.clusters(train_per_cloud, 8, seed + 20000 + i, dtype=dt, centres=centres, sigmas=sig)
        out[dt][0].append(cloud)
        out[dt][1].append(qs)
        out[dt][2].append(tr)
    return out


def run_c4(args):
    import torch

    import libnabo_gb300 as nb
    from oracle import oracle as O

    from libnabo_gb300 import autotune

    dev = torch.device("cuda", 0)
    data = c4_workload(args.c4_clouds)
    k = 32
    batches = []
    t_gen = time.perf_counter()
    for dt, (clouds, queries, train_queries) in data.items():
        if not clouds:
            continue
        pc = np.array([c.shape[0] for c in clouds], np.int64)
        qc = np.array([q.shape[0] for q in queries], np.int64)
        # the autotuner on 4 clouds, 25,000 queries each; one thread per
        # query (8-lane groups measured 6-8x slower on these batches)
        t0 = time.perf_counter()
        choice = autotune.tune(clouds, queries, k, dim=8, dtype=dt, sample=4, repeats=2,
                               split_rules=tuple(int(r) for r in args.split_rules.split(",")),
                               max_queries_per_cloud=25000, lanes=(1,))
        choice["autotune_s"] = time.perf_counter() - t0
        b = nb.BatchSearch(pc, dim=8, dtype=dt, bucketSize=choice["bucketSize"],
                           threadsPerBlock=choice["threadsPerBlock"], maxLevels=choice["maxLevels"],
                           splitRule=choice["splitRule"])
        b.set_queries(qc, np.full(len(clouds), k, np.int32))
        tc = torch.from_numpy(np.concatenate(clouds)).to(dev)
        tq = torch.from_numpy(np.concatenate(queries)).to(dev)
        batches.append(dict(dt=dt, b=b, tc=tc, tq=tq, out=b._outputs(dev), clouds=clouds, queries=queries,
                            train_queries=train_queries, points=int(pc.sum()), nq=int(qc.sum()),
                            choice={kk: choice[kk] for kk in ("bucketSize", "threadsPerBlock", "splitRule",
                                                              "maxLevels", "autotune_s")}))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for x in batches:
        x["b"].build(x["tc"])
    e1.record()
    torch.cuda.synchronize()
    build_ms = e0.elapsed_time(e1)
    for x in batches:  # a tree deeper than 64 top levels: rebuild with room for it
        if x["b"].status()["flags"] & 2:
            x["b"] = nb.BatchSearch([c.shape[0] for c in x["clouds"]], dim=8, dtype=x["dt"],
                                    bucketSize=x["choice"]["bucketSize"],
                                    threadsPerBlock=x["choice"]["threadsPerBlock"], maxLevels=256,
                                    splitRule=x["choice"]["splitRule"])
            x["b"].set_queries([q.shape[0] for q in x["queries"]], np.full(len(x["clouds"]), k, np.int32))
            x["b"].build(x["tc"])
    status = {np.dtype(x["dt"]).name: x["b"].status() for x in batches}
    nq_total = sum(x["nq"] for x in batches)

    def step(eps, outs=None):
        for j, x in enumerate(batches):
            x["b"].knn(x["tq"], epsilon=eps, out=outs[j] if outs else x["out"])

    forms = {}
    exact_out = None
    with ClockSampler(0) as clk:
        for eps in (0.0, 0.5):
            outs = [x["b"]._outputs(dev) for x in batches]
            for _ in range(args.warmup):
                step(eps, outs)
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
            for a0, a1 in ev:
                a0.record()
                step(eps, outs)
                a1.record()
            torch.cuda.synchronize()
            ms = sum(a0.elapsed_time(a1) for a0, a1 in ev) / args.steps
            forms[f"eps{eps}"] = {"ms_per_step": ms, "queries_per_s": nq_total / (ms / 1e3)}
            if eps == 0.0:
                exact_out = outs
            else:
                approx_out = outs
    # per scalar type, exact search
    per_type = {}
    for j, x in enumerate(batches):
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        x["b"].knn(x["tq"], epsilon=0.0, out=exact_out[j])
        a1.record()
        torch.cuda.synchronize()
        ms = a0.elapsed_time(a1)
        per_type[np.dtype(x["dt"]).name] = {"ms": ms, "queries_per_s": x["nq"] / (ms / 1e3)}
    forms["eps0.0"]["per_type"] = per_type
    # learned-radius form: one network per (dimension, scalar type), trained
    # on queries disjoint from the timed ones (fresh draws from each cloud's
    # mixture) with exact distances from the plain batched search
    learned = None
    if not args.no_learned:
        learned = {}
        t_train = time.perf_counter()
        for x in batches:
            b = x["b"]
            trq = x["train_queries"]
            b.set_queries([q.shape[0] for q in trq], np.full(len(x["clouds"]), k, np.int32))
            tt = torch.from_numpy(np.concatenate(trq)).to(dev)
            _, td2 = b.knn(tt)
            x["model"] = b.train_radius_model(tt, td2)
            b.set_queries([q.shape[0] for q in x["queries"]], np.full(len(x["clouds"]), k, np.int32))
            x["train_n"] = int(tt.shape[0])
            del tt, td2
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t_train
        fbs = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in batches]

        def lstep(eps, outs):
            for j, x in enumerate(batches):
                fbs[j].zero_()
                x["b"].knn_learned(x["model"], x["tq"], epsilon=eps, out=outs[j], fallbacks=fbs[j])

        for eps in (0.0, 0.5):
            outs = [x["b"]._outputs(dev) for x in batches]
            for _ in range(args.warmup):
                lstep(eps, outs)
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            for a0, a1 in ev:
                a0.record()
                lstep(eps, outs)
                a1.record()
            torch.cuda.synchronize()
            ms = sum(a0.elapsed_time(a1) for a0, a1 in ev) / args.steps
            entry = {"ms_per_step": ms, "queries_per_s": nq_total / (ms / 1e3),
                     "fallbacks": int(sum(int(f.item()) for f in fbs)),
                     "fallback_rate": sum(int(f.item()) for f in fbs) / nq_total}
            if eps == 0.0:
                entry["identical_to_plain"] = bool(all(
                    torch.equal(outs[j][0], exact_out[j][0]) and torch.equal(outs[j][1], exact_out[j][1])
                    for j in range(len(batches))))
            else:
                entry["within_bound_of_exact"] = bool(all(
                    bool((outs[j][1] <= (1.5 ** 2) * exact_out[j][1] * (1 + 1e-6)).all())
                    for j in range(len(batches))))
            learned[f"eps{eps}"] = entry
        learned["models"] = {np.dtype(x["dt"]).name: dict(x["model"].meta, train_queries=x["train_n"])
                             for x in batches}

        # where the time goes, per scalar type (best of 2, epsilon 0): the
        # plain search, the learned search, its network alone, and the bound
        # of any radius predictor -- each query's exact k-th distance (a hair
        # above) as its radius
        def t_best(fn, reps=2):
            best = float("inf")
            for _ in range(reps):
                torch.cuda.synchronize()
                a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a0.record()
                fn()
                a1.record()
                torch.cuda.synchronize()
                best = min(best, a0.elapsed_time(a1))
            return best

        parts = {}
        for j, x in enumerate(batches):
            b, tq = x["b"], x["tq"]
            tmp = b._outputs(dev)
            dk2 = exact_out[j][1].view(-1, k)[:, -1]
            ideal = (torch.sqrt(dk2) * (1 + 2.0 ** -20)).to(dk2.dtype).contiguous()
            entry = {"plain_ms": t_best(lambda: b.knn(tq, out=tmp)),
                     "learned_ms": t_best(lambda: b.knn_learned(x["model"], tq, out=tmp)),
                     "network_ms": t_best(lambda: b.predict_radii(x["model"], tq)),
                     "ideal_radius_ms": t_best(lambda: b.knn_radii(tq, ideal, out=tmp))}
            entry["ideal_radius_identical"] = bool(torch.equal(tmp[0], exact_out[j][0])
                                                   and torch.equal(tmp[1], exact_out[j][1]))
            parts[np.dtype(x["dt"]).name] = entry
        learned["per_type_eps0"] = parts
        learned["train_s"] = train_s
        learned["train_queries_from"] = "fresh draws from each cloud's mixture, disjoint from the timed queries"
    forms["learned"] = learned
    # CPU baseline: the oracle (reference algorithm, all host threads) on the
    # two smallest clouds of each type, 5,000 queries each
    base = None
    if not args.no_cpu_baseline:
        nqb, tb, touched = 0, 0.0, 0
        for x in batches:
            for c in np.argsort([cl.shape[0] for cl in x["clouds"]])[:2]:
                qs = x["queries"][c][:5000]
                tree = O.OracleTree(x["clouds"][c], creation_flags=O.TOUCH_STATISTICS)
                t0 = time.perf_counter()
                _, _, tcount = tree.knn(qs, k, mode=O.MODE_REFERENCE)
                tb += time.perf_counter() - t0
                nqb += qs.shape[0]
                touched += int(tcount)
        base = {"value": nqb / tb, "unit": "queries/s", "cores": O.num_threads(), "kind": "port",
                "sample": f"search only, 2 smallest clouds of each type, 5000 queries each ({nqb} queries, eps 0)",
                "touched_per_query": touched / nqb}
    # checks on the smallest cloud of each type: exact at eps 0 (the
    # oracle's tree in canonical order for the reference's split rule, its
    # brute force for the median split), the (1+eps)^2 bound on squared
    # distances at eps 0.5
    checks = {}
    for j, x in enumerate(batches):
        c = int(np.argmin([cl.shape[0] for cl in x["clouds"]]))
        sub = slice(0, 2000)
        gi = x["b"].split(exact_out[j][0].cpu().numpy())[c][sub]
        gd = x["b"].split(exact_out[j][1].cpu().numpy())[c][sub]
        ad = x["b"].split(approx_out[j][1].cpu().numpy())[c][sub]
        if x["choice"]["splitRule"] == 1:
            oi, od, _ = O.bf_knn(x["clouds"][c], x["queries"][c][sub], k, mode=O.MODE_CANONICAL)
        else:
            oi, od, _ = O.OracleTree(x["clouds"][c]).knn(x["queries"][c][sub], k, mode=O.MODE_CANONICAL)
        checks[np.dtype(x["dt"]).name] = {
            "cloud": c, "points": int(x["clouds"][c].shape[0]), "queries_checked": 2000,
            "exact_identical": bool(np.array_equal(gi, oi) and np.array_equal(gd, od)),
            "eps0.5_within_bound": bool((ad <= (1.5 ** 2) * od * (1 + 1e-6)).all())}
    res = {
        "metric": C4_METRIC, "value": forms["eps0.0"]["queries_per_s"], "unit": "queries/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": forms["eps0.0"]["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "c4_8d", "clouds": sum(len(x["clouds"]) for x in batches),
                   "points": sum(x["points"] for x in batches), "queries": nq_total, "k": k, "dims": 8,
                   "per_type": {np.dtype(x["dt"]).name: {"clouds": len(x["clouds"]), "points": x["points"],
                                                          "queries": x["nq"], "autotuned": x["choice"]}
                                for x in batches},
                   "step": "search of every query of both batches (trees built once)",
                   "l2": "inputs larger than L2"},
        "forms": forms, "build_ms": build_ms, "status": status, "checks": checks, "cpu_baseline": base,
        "clocks": clk.summary(), "data_s": time.perf_counter() - t_gen,
    }
    print(json.dumps(res, default=str))


# ---------------------------------------------------------------------------
# Brute force: 100,000 uniform 3-D float32 points against 100,000 queries,
# k = 5 (the reference's small case scaled up so one launch is measurable).
# Bound by the FP32 pipe: flops = Q * N * 3D (D subtractions and D
# multiply-adds counted as two), against the FMA peak measured live.

BF_METRIC = "brute-force kNN queries/s (100k uniform 3-D points, k=5)"


def run_bf(args):
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import synthetic as S
    from oracle import oracle as O

    dev = torch.device("cuda", 0)
    n, nq, k, d = 100_000, 100_000, 5, 3
    cloud = S.uniform(n, d, seed=S.SEED_BASE + 9)
    q = S.uniform(nq, d, seed=S.SEED_BASE + 10)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA)
    tq = torch.from_numpy(q).to(dev)
    idx = torch.empty((nq, k), dtype=torch.int32, device=dev)
    d2 = torch.empty((nq, k), dtype=torch.float32, device=dev)
    s.profile(True)
    for _ in range(args.warmup):
        s.knn_device(tq, k, out=(idx, d2))
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kms = []
    with ClockSampler(0) as clk:
        for e0, e1 in ev:
            e0.record()
            s.knn_device(tq, k, out=(idx, d2))
            e1.record()
            kms.append(s.last_kernel_ms())
        torch.cuda.synchronize()
    step_ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / args.steps
    kernel_ms = statistics.mean(kms)
    peak = nb.measure_fma_peak(np.float32)
    flops = float(nq) * n * 3 * d
    achieved = flops / (kernel_ms * 1e-3)
    # exactness and CPU baseline on a sample of the queries
    sample = 2000
    t0 = time.perf_counter()
    oi, od, _ = O.bf_knn(cloud, q[:sample], k, mode=O.MODE_CANONICAL)
    cpu_s = time.perf_counter() - t0
    gi = idx[:sample].cpu().numpy()
    gd = d2[:sample].cpu().numpy()
    hi, hd = s.knn(q, k)  # host API, for e2e
    t0 = time.perf_counter()
    for _ in range(3):
        s.knn(q, k)
    e2e_s = (time.perf_counter() - t0) / 3
    res = {
        "metric": BF_METRIC, "value": nq / (step_ms / 1e3), "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "bruteforce_uniform_100k_k5", "points": n, "queries": nq, "k": k,
                   "l2": "cloud (1.6 MB) is reread from L2 by design; the bound is the FP32 pipe"},
        "e2e": {"value": nq / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                "d2h_bytes_per_step": int(nq * k * 8)},
        "roofline": {"bound": "fp32 pipe", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": "FMA chains measured in this run",
                     "kernel": "k_knn_bruteforce", "kernel_ms": kernel_ms, "flops_per_launch": flops},
        "exact_vs_oracle": {"queries_checked": sample,
                            "identical": bool(np.array_equal(gi, oi) and np.array_equal(gd, od))},
        "cpu_baseline": {"value": sample / cpu_s, "unit": "queries/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"{sample} queries against all {n} points (oracle brute force)"},
        "clocks": clk.summary(), "gpu_launches": args.steps,
    }
    # the same search in double: bound by the FP64 pipe (1/64 of the FP32
    # rate on this GPU), so fewer queries
    nq64 = 20_000
    cloud64, q64 = cloud.astype(np.float64), q[:nq64].astype(np.float64)
    s64 = nb.NearestNeighbourSearch(cloud64, nb.SearchType.BRUTE_FORCE_CUDA)
    tq64 = torch.from_numpy(q64).to(dev)
    idx64 = torch.empty((nq64, k), dtype=torch.int32, device=dev)
    d264 = torch.empty((nq64, k), dtype=torch.float64, device=dev)
    s64.profile(True)
    for _ in range(args.warmup):
        s64.knn_device(tq64, k, out=(idx64, d264))
    torch.cuda.synchronize()
    kms64 = []
    for _ in range(args.steps):
        s64.knn_device(tq64, k, out=(idx64, d264))
        kms64.append(s64.last_kernel_ms())
    torch.cuda.synchronize()
    kernel64 = statistics.mean(kms64)
    peak64 = nb.measure_fma_peak(np.float64)
    flops64 = float(nq64) * n * 3 * d
    oi64, od64, _ = O.bf_knn(cloud64, q64[:500], k, mode=O.MODE_CANONICAL)
    res["f64"] = {"queries": nq64, "points": n, "k": k, "kernel_ms": kernel64, "value": nq64 / (kernel64 / 1e3),
                  "unit": "queries/s", "achieved_tflops": flops64 / (kernel64 * 1e-3) / 1e12,
                  "peak_tflops": peak64 / 1e12, "frac": flops64 / (kernel64 * 1e-3) / peak64,
                  "peak_source": "FP64 FMA chains measured in this run",
                  "identical_vs_oracle": bool(np.array_equal(idx64[:500].cpu().numpy(), oi64)
                                              and np.array_equal(d264[:500].cpu().numpy(), od64))}
    print(json.dumps(res))


def run_latency(args):
    """Per-call latency of the host-buffer API (the reference's knn on host
    matrices, nabo/nabo.h:338, and its single-point form, nabo/nabo.h:325)
    for batches of 1 to 65,536 lidar queries, k=10, r = 1 m; the oracle
    (the reference algorithm, all host threads) timed the same way."""
    import libnabo_gb300 as nb
    from libnabo_gb300 import synthetic as S
    from oracle import oracle as O

    cloud = S.lidar_scan()
    q = S.lidar_queries(cloud)
    k, r = 10, 1.0
    import torch
    s = nb.NearestNeighbourSearch(cloud)
    sp = nb.NearestNeighbourSearch(cloud)  # device API with the kernel bracketed by events
    sp.profile(True)
    orc = O.OracleTree(cloud)
    sizes = [1, 16, 256, 4096, 65536]
    rows = {}
    with ClockSampler(0) as clk:
        for n in sizes:
            qq = np.ascontiguousarray(q[:n])
            tq = torch.from_numpy(qq).cuda()
            kms = []
            for i in range(25):
                sp.knn_device(tq, k, 0.0, 0, r)
                if i >= 5:
                    kms.append(sp.last_kernel_ms())
            reps = max(20, min(2000, 400_000 // n))
            for _ in range(max(args.warmup, 5)):
                gi, gd = s.knn(qq, k, 0.0, 0, r)
            t = []
            for _ in range(reps):
                t0 = time.perf_counter()
                s.knn(qq, k, 0.0, 0, r)
                t.append(time.perf_counter() - t0)
            oi, od, _ = orc.knn(qq, k, 0.0, 0, r, mode=O.MODE_CANONICAL)
            tc = []
            for _ in range(min(reps, 200)):
                t0 = time.perf_counter()
                orc.knn(qq, k, 0.0, 0, r, mode=O.MODE_CANONICAL)
                tc.append(time.perf_counter() - t0)
            g_us = statistics.median(t) * 1e6
            c_us = statistics.median(tc) * 1e6
            rows[str(n)] = {"gpu_us_per_call": g_us, "gpu_queries_per_s": n / (g_us * 1e-6),
                            "search_kernel_us": statistics.median(kms) * 1e3,
                            "cpu_us_per_call": c_us, "cpu_queries_per_s": n / (c_us * 1e-6),
                            "calls_timed": reps,
                            "identical": bool(np.array_equal(gi, oi) and np.array_equal(gd, od))}
    one = rows["1"]
    res = {
        "metric": "host-API kNN call latency, one query (lidar 1.15M points, k=10)", "value": one["gpu_us_per_call"],
        "unit": "us", "n_gpus": 1, "steps": None, "warmup": max(args.warmup, 5), "ms_per_step": one["gpu_us_per_call"] / 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "latency_lidar64_k10", "points": int(cloud.shape[0]), "k": k, "maxRadius": r,
                   "timing": "median wall time of the Python call (ctypes) from host arrays to host arrays, "
                             "both arms; the GPU arm includes the copies and the stream synchronisation"},
        "sizes": rows,
        "cpu_baseline": {"value": one["cpu_us_per_call"], "unit": "us", "cores": O.num_threads(), "kind": "port",
                         "sample": "the same calls on the oracle"},
        "clocks": clk.summary(), "gpu_launches": 1,
    }
    print(json.dumps(res))


def run_batched_reference(args):
    """The reference algorithm (oracle restatement, all host threads) on a
    sample of the batched workload's clouds; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    clouds, queries, ks = batched_workload(0)
    for _ in range(args.warmup):
        batched_cpu(clouds, queries, ks, sample=4, seed=99)
    vals = [batched_cpu(clouds, queries, ks) for _ in range(args.steps)]
    v = statistics.mean(x["value"] for x in vals)
    base = vals[0]
    nq = sum(queries[c].shape[0] for c in base["clouds"])
    out = {
        "metric": BATCH_METRIC, "value": v, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": nq / v * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": "batched512_3d", "search": "KDTREE_LINEAR_HEAP restated in C++/OpenMP "
                   "(oracle/nabo_oracle.cpp), tree build + search per cloud"},
        "cpu_baseline": {"value": v, "unit": "queries/s", "cores": base["cores"], "kind": "port",
                         "sample": base["sample"]},
        "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def max_ranks(x, world):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def main():
    args = parse()
    if args.impl == "reference" and args.workload in ("c4", "bf", "latency"):
        # these workloads time the reference algorithm on the host cores
        # themselves (the cpu_baseline field of their line)
        print(json.dumps({"impl": "reference", "workload": args.workload,
                          "unavailable": "no separate reference arm for this workload: its own line reports the "
                                         "reference algorithm on the host cores in cpu_baseline"}))
        return
    if args.workload == "c4":
        run_c4(args)
        return
    if args.workload == "bf":
        run_bf(args)
        return
    if args.workload == "latency":
        run_latency(args)
        return
    if args.workload == "batched":
        if args.impl == "reference":
            run_batched_reference(args)
        else:
            run_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
