"""Multi-rank split of a search (libnabo_gb300.sharding) on CPU: query ranges,
cost-balanced cloud assignment, and two gloo ranks whose gathered results equal
the single-process ones. The per-rank search is the oracle (the GPU search
takes the same place on a multi-GPU node)."""
import os
import socket

import numpy as np
import pytest

from libnabo_gb300 import sharding as SH


def test_query_ranges_cover_in_order():
    for nq, world in ((0, 2), (1, 2), (10, 3), (1000, 8), (7, 7)):
        r = SH.query_ranges(nq, world)
        assert len(r) == world and r[0][0] == 0 and r[-1][1] == nq
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        sizes = [h - l for l, h in r]
        assert max(sizes) - min(sizes) <= 1


def test_balance_clouds_assigns_each_once_and_balances():
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(0, 6, 300))
    for world in (1, 2, 4, 8):
        parts, load = SH.balance_clouds(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(costs.shape[0]))
        # greedy LPT: no rank exceeds the mean load by more than the largest cost
        assert max(load) <= costs.sum() / world + costs.max() + 1e-9
        for p, l in zip(parts, load):
            assert abs(costs[p].sum() - l) < 1e-6 * max(l, 1.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, cloud, queries, k, out_path):
    import torch.distributed as dist

    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    O.set_threads(1)
    tree = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)

    def search(block):
        return tree.knn(block, k, mode=O.MODE_CANONICAL)

    idx, d2, touched = SH.search_sharded(search, queries, k, rank, world)
    # batches: clouds split by cost, every rank ends up with every result
    clouds = [cloud[: 500 + 300 * c] for c in range(5)]
    qs = [queries[: 200 + 50 * c] for c in range(5)]
    ks = [1, 4, k, 2, 3]

    def search_clouds(mine):
        return {c: O.OracleTree(clouds[c]).knn(qs[c], ks[c], mode=O.MODE_CANONICAL)[:2] for c in mine}

    res = SH.batch_sharded(search_clouds, [c.shape[0] for c in clouds], [q.shape[0] for q in qs], ks, rank, world)
    if rank == 0:
        np.savez(out_path, idx=idx, d2=d2, touched=touched,
                 **{f"b{c}_i": res[c][0] for c in res}, **{f"b{c}_d": res[c][1] for c in res})
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path):
    import multiprocessing as mp

    from libnabo_gb300 import synthetic as S
    from oracle import oracle as O
    cloud = S.uniform(4000, 3, seed=11)
    queries = S.uniform(1001, 3, seed=12)  # odd: ranges of unequal size
    k = 6
    out = str(tmp_path / "rank0.npz")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, cloud, queries, k, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = np.load(out)
    ref_i, ref_d, ref_t = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS).knn(queries, k,
                                                                                     mode=O.MODE_CANONICAL)
    assert np.array_equal(got["idx"], ref_i) and np.array_equal(got["d2"], ref_d)
    assert int(got["touched"]) == int(ref_t)
    clouds = [cloud[: 500 + 300 * c] for c in range(5)]
    qs = [queries[: 200 + 50 * c] for c in range(5)]
    ks = [1, 4, k, 2, 3]
    for c in range(5):
        oi, od, _ = O.OracleTree(clouds[c]).knn(qs[c], ks[c], mode=O.MODE_CANONICAL)
        assert np.array_equal(got[f"b{c}_i"], oi) and np.array_equal(got[f"b{c}_d"], od)


def test_single_rank_is_plain_search():
    from oracle import oracle as O
    from libnabo_gb300 import synthetic as S
    cloud = S.uniform(1000, 3, seed=3)
    q = S.uniform(100, 3, seed=4)
    tree = O.OracleTree(cloud)
    i, d, t = SH.search_sharded(lambda b: tree.knn(b, 3), q, 3, 0, 1)
    ri, rd, rt = tree.knn(q, 3)
    assert np.array_equal(i, ri) and np.array_equal(d, rd)
