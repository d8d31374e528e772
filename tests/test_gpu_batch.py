"""Batches of uneven clouds: one forest build, one search launch, CUDA-graph
replay and the autotuner -- against single-cloud searches and the oracle."""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def _batch_data(n_clouds, lo, hi, seed, dtype=np.float32):
    from libnabo_gb300 import synthetic as S
    sizes = S.log_uniform_sizes(n_clouds, lo, hi, seed)
    sizes[:4] = [3, 9, 200, 300][: min(4, n_clouds)]  # single bucket, tiny, below and above the top-phase size
    rng = np.random.default_rng(seed + 1)
    clouds = [S.gaussian_blobs(int(n), seed + 10 + i, dtype=dtype) for i, n in enumerate(sizes)]
    queries = [(c + rng.normal(0, 0.01, c.shape)).astype(dtype) for c in clouds]
    ks = rng.choice([1, 5, 16], n_clouds).astype(np.int32)
    ks = np.minimum(ks, sizes - 1).astype(np.int32)
    return clouds, queries, ks


def _run_batch(clouds, queries, ks, dtype=np.float32, graph=False, **kw):
    import torch
    nb = _nb()
    b = nb.BatchSearch([c.shape[0] for c in clouds], dim=clouds[0].shape[1], dtype=dtype, **kw)
    b.set_queries([q.shape[0] for q in queries], ks)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    if graph:
        idx, d2 = b.run(tc, tq)
    else:
        b.build(tc)
        idx, d2 = b.knn(tq)
    torch.cuda.synchronize()
    return b, b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())


def test_batch_trees_equal_oracle_trees():
    clouds, queries, ks = _batch_data(40, 300, 30000, seed=1)
    b, _, _ = _run_batch(clouds, queries, ks)
    st = b.status()
    assert st["ok"], st
    for c, cloud in enumerate(clouds):
        g = b.export_tree(c)
        o = O.OracleTree(cloud).export()
        for key in ("cut_dim", "right", "bucket_start", "bucket_count", "buckets"):
            assert np.array_equal(g[key], o[key]), (c, key)
        inner = o["cut_dim"] >= 0
        assert np.array_equal(g["cut_val"][inner], o["cut_val"][inner]), c


@pytest.mark.parametrize("graph", [False, True])
def test_large_batch_trees_equal_oracle_trees(graph):
    """A forest of 4.8 M points (about 37 k small segments, one warp each,
    many more than the warps resident at once)."""
    from libnabo_gb300 import synthetic as S
    sizes = [120_000] * 40
    clouds = [S.gaussian_blobs(n, 900 + i) for i, n in enumerate(sizes)]
    queries = [c[:100] for c in clouds]
    ks = np.full(len(clouds), 4, np.int32)
    b, gi, gd = _run_batch(clouds, queries, ks, graph=graph, maxLevels=64)
    assert b.status()["ok"], b.status()
    for c in (0, 17, 39):
        g = b.export_tree(c)
        o = O.OracleTree(clouds[c]).export()
        for key in ("cut_dim", "right", "bucket_start", "bucket_count", "buckets"):
            assert np.array_equal(g[key], o[key]), (c, key)
        oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], 4, mode=O.MODE_CANONICAL)
        H.assert_identical(gi[c], gd[c], oi, od, f"cloud {c}")


@pytest.mark.parametrize("graph", [False, True])
def test_batch_results_equal_single_searches(graph):
    nb = _nb()
    clouds, queries, ks = _batch_data(60, 300, 40000, seed=2)
    b, bi, bd = _run_batch(clouds, queries, ks, graph=graph)
    assert b.status()["ok"]
    for c, (cloud, q) in enumerate(zip(clouds, queries)):
        s = nb.NearestNeighbourSearch(cloud)
        si, sd = s.knn(q, int(ks[c]))
        H.assert_identical(bi[c], bd[c], si, sd, f"cloud {c} (n={cloud.shape[0]}, k={ks[c]})")
        if c < 8:
            oi, od, _ = O.OracleTree(cloud).knn(q, int(ks[c]), mode=O.MODE_CANONICAL)
            H.assert_identical(bi[c], bd[c], oi, od, f"cloud {c} vs oracle")


def test_graph_replay_follows_new_data():
    import torch
    nb = _nb()
    clouds, queries, ks = _batch_data(30, 300, 20000, seed=3)
    b = nb.BatchSearch([c.shape[0] for c in clouds])
    b.set_queries([q.shape[0] for q in queries], ks)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    out = b._outputs(tq.device)
    b.run(tc, tq, out=out)
    torch.cuda.synchronize()
    first = [x.copy() for x in b.split(out[0].cpu().numpy())]
    # new coordinates of the same shapes written into the captured buffers
    clouds2, queries2, _ = _batch_data(30, 300, 20000, seed=33)
    clouds2 = [np.resize(c2, c.shape).astype(np.float32) for c, c2 in zip(clouds, clouds2)]
    queries2 = [(c + 0.01).astype(np.float32) for c in clouds2]
    tc.copy_(torch.from_numpy(np.concatenate(clouds2)).cuda())
    tq.copy_(torch.from_numpy(np.concatenate(queries2)).cuda())
    b.run(tc, tq, out=out)
    torch.cuda.synchronize()
    second_i = b.split(out[0].cpu().numpy())
    second_d = b.split(out[1].cpu().numpy())
    changed = 0
    for c in range(len(clouds)):
        oi, od, _ = O.OracleTree(clouds2[c]).knn(queries2[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(second_i[c], second_d[c], oi, od, f"replay cloud {c}")
        changed += int(not np.array_equal(first[c], second_i[c]))
    assert changed > 0


@pytest.mark.parametrize("graph", [False, True])
def test_level_limit_is_reported_and_search_stays_exact(graph):
    """Too few levels for the clouds: the build reports it, and every cloud
    becomes one leaf, so the same launch still returns exact neighbours."""
    clouds, queries, ks = _batch_data(8, 2000, 6000, seed=4)
    b, bi, bd = _run_batch(clouds, queries, ks, graph=graph, maxLevels=2)
    st = b.status()
    assert not st["ok"] and (st["flags"] & 2), st
    assert st["nodes"] == len(clouds) and st["height"] == 0, st
    for c in (0, 3, 7):
        oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(bi[c], bd[c], oi, od, f"level-limited cloud {c}")


def test_non_finite_batch_is_reported():
    nb = _nb()
    import torch
    clouds, queries, ks = _batch_data(5, 1000, 2000, seed=5)
    clouds[3][7, 0] = np.nan
    b = nb.BatchSearch([c.shape[0] for c in clouds])
    b.set_queries([q.shape[0] for q in queries], ks)
    b.build(torch.from_numpy(np.concatenate(clouds)).cuda())
    assert b.status()["flags"] & 1


def test_autotuner_choice_is_exact():
    nb = _nb()
    from libnabo_gb300 import autotune
    clouds, queries, ks = _batch_data(48, 2000, 60000, seed=6)
    choice = autotune.tune(clouds, queries, ks, sample=16, repeats=2)
    assert choice["bucketSize"] in autotune.CANDIDATES["bucketSize"]
    assert {t["splitRule"] for t in choice["trials"]} == {0, 1}
    assert {t["lanesPerQuery"] for t in choice["trials"]} == {1, 8}
    b, bi, bd = _run_batch(clouds, queries, ks, graph=True, bucketSize=choice["bucketSize"],
                           threadsPerBlock=choice["threadsPerBlock"], maxLevels=choice["maxLevels"],
                           splitRule=choice["splitRule"], lanesPerQuery=choice["lanesPerQuery"])
    assert b.status()["ok"]
    for c in range(0, len(clouds), 7):
        # the reference's tree (split rule 0) or the median-split tree (1):
        # either returns the exact k smallest pairs
        oi, od, _ = O.bf_knn(clouds[c], queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(bi[c], bd[c], oi, od, f"tuned cloud {c}")
    # restricted to the reference's trees on request
    ref_only = autotune.tune(clouds, queries, ks, sample=8, repeats=1, split_rules=(0,))
    assert ref_only["splitRule"] == 0
    again = autotune.tune(clouds, queries, ks, sample=16, repeats=2)
    assert again["cached"]


def _host_buffers(pinned):
    """Copies of arrays in page-locked (pinned=True) or ordinary host memory;
    the pinned tensors stay referenced by the returned list."""
    import torch
    hold = []

    def host(a):
        a = np.ascontiguousarray(a)
        if not pinned:
            return a.copy()
        t = torch.from_numpy(a).pin_memory()
        hold.append(t)
        return t.numpy()
    return host, hold


def _device_flat(b, clouds, queries, **kw):
    """The device-buffer run (graph) of batch b: flat host copies of its results."""
    import torch
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    idx, d2 = b.run(tc, tq, **kw)
    torch.cuda.synchronize()
    return idx.cpu().numpy(), d2.cpu().numpy()


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_host_run_equals_device_run(pinned, dtype):
    """nabo_cuda_batch_run_host: same results as the device run, replays on
    new data written into the same host buffers, recaptures on new
    arguments; one cloud without queries."""
    nb = _nb()
    clouds, queries, ks = _batch_data(50, 300, 30000, seed=5, dtype=dtype)
    queries[7] = queries[7][:0]
    b = nb.BatchSearch([c.shape[0] for c in clouds], dtype=dtype)
    b.set_queries([q.shape[0] for q in queries], ks)
    host, hold = _host_buffers(pinned)
    hc, hq = host(np.concatenate(clouds)), host(np.concatenate(queries))
    out = (host(np.full(b.result_entries, -7, np.int32)), host(np.full(b.result_entries, -1, dtype)))
    gi, gd = b.run_host(hc, hq, out=out)
    assert gi is out[0] and gd is out[1]
    di, dd = _device_flat(b, clouds, queries)
    H.assert_identical(gi[:, None], gd[:, None], di[:, None], dd[:, None], "host run vs device run")
    for c in (0, 1, 7, 20, 49):
        oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(b.split(gi)[c], b.split(gd)[c], oi, od, f"cloud {c}")
    # new coordinates in the same buffers: the captured graph reads them
    clouds2 = [(c * 1.5 + 0.25).astype(dtype) for c in clouds]
    queries2 = [(q * 1.5 + 0.25).astype(dtype) for q in queries]
    hc[:] = np.concatenate(clouds2)
    hq[:] = np.concatenate(queries2)
    gi, gd = b.run_host(hc, hq, out=out)
    for c in (0, 3, 33):
        oi, od, _ = O.OracleTree(clouds2[c]).knn(queries2[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(b.split(gi)[c], b.split(gd)[c], oi, od, f"replay cloud {c}")
    # another radius: a new capture, same results as the device run
    gi, gd = b.run_host(hc, hq, maxRadius=0.02, out=out)
    di, dd = _device_flat(b, clouds2, queries2, maxRadius=0.02)
    H.assert_identical(gi[:, None], gd[:, None], di[:, None], dd[:, None], "host run with a radius")
    assert (gi == -1).any() and (gi >= 0).any()
    del hold


@pytest.mark.parametrize("chunks", [1, 3, 64])
def test_host_run_groups_and_wide_k(chunks):
    """Cloud groups of the pinned host run (one, three, more groups than
    clouds), with a cloud whose k sends the batch to the warp-per-query
    kernel."""
    nb = _nb()
    clouds, queries, _ = _batch_data(12, 300, 5000, seed=6)
    rng = np.random.default_rng(6)
    ks = np.minimum(rng.choice([1, 5, 40], len(clouds)), [c.shape[0] - 1 for c in clouds]).astype(np.int32)
    ks[5] = min(40, clouds[5].shape[0] - 1)
    b = nb.BatchSearch([c.shape[0] for c in clouds], pipelineChunks=chunks)
    b.set_queries([q.shape[0] for q in queries], ks)
    host, hold = _host_buffers(True)
    hc, hq = host(np.concatenate(clouds)), host(np.concatenate(queries))
    out = (host(np.zeros(b.result_entries, np.int32)), host(np.zeros(b.result_entries, np.float32)))
    gi, gd = b.run_host(hc, hq, out=out)
    for c in range(len(clouds)):
        oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(b.split(gi)[c], b.split(gd)[c], oi, od, f"cloud {c} k={ks[c]}")
    del hold


def test_host_run_argument_errors():
    nb = _nb()
    clouds, queries, ks = _batch_data(6, 300, 2000, seed=7)
    b = nb.BatchSearch([c.shape[0] for c in clouds])
    with pytest.raises(nb.NaboError, match="set_queries"):
        b.run_host(np.concatenate(clouds), np.concatenate(queries))
    b.set_queries([q.shape[0] for q in queries], ks)
    with pytest.raises(nb.NaboError, match="clouds must be"):
        b.run_host(np.concatenate(clouds)[1:], np.concatenate(queries))
    with pytest.raises(nb.NaboError, match="self match"):
        b.run_host(np.concatenate(clouds), np.concatenate(queries), optionFlags=nb.ALLOW_SELF_MATCH)
    with pytest.raises(nb.NaboError, match="pipelineChunks"):
        nb.BatchSearch([c.shape[0] for c in clouds], pipelineChunks=65)


@pytest.mark.parametrize("graph", [False, True])
def test_lane_groups_per_query_are_exact(graph):
    """Batches searched by 8-lane groups per query (k <= 32) return the
    one-thread-per-query results."""
    clouds, queries, ks = _batch_data(20, 300, 20000, seed=12)
    _, bi, bd = _run_batch(clouds, queries, ks, graph=graph, lanesPerQuery=8)
    _, ri, rd = _run_batch(clouds, queries, ks, graph=graph)
    for c in range(len(clouds)):
        H.assert_identical(bi[c], bd[c], ri[c], rd[c], f"lane groups cloud {c}")


@pytest.mark.parametrize("split_rule", [0, 1])
@pytest.mark.parametrize("chunks", [1, 3, 5])
def test_k_size_launches_with_mixed_k_and_empty_clouds(split_rule, chunks):
    """The search runs one launch per compiled top-k size (1, 2, 5, 8, 10,
    16, 32) over run lists of its clouds. Clouds whose k is below their
    group's size (3 and 4 in the 5-slot group, 9 in the 10-slot one),
    clouds without queries (no run), and host runs whose cloud groups cut
    every size's run list must all give the oracle's results."""
    nb = _nb()
    clouds, queries, _ = _batch_data(22, 300, 8000, seed=11)
    ks = np.array([1, 2, 3, 5, 4, 7, 8, 9, 10, 12, 16, 20, 32, 1, 5, 16, 3, 9, 32, 2, 8, 10], np.int32)
    ks = np.minimum(ks, [c.shape[0] - 1 for c in clouds]).astype(np.int32)
    for c in (4, 13, 21):
        queries[c] = queries[c][:0]
    b = nb.BatchSearch([c.shape[0] for c in clouds], splitRule=split_rule, pipelineChunks=chunks, maxLevels=40)
    b.set_queries([q.shape[0] for q in queries], ks)
    di, dd = _device_flat(b, clouds, queries)
    host, hold = _host_buffers(True)
    hc, hq = host(np.concatenate(clouds)), host(np.concatenate(queries))
    out = (host(np.zeros(b.result_entries, np.int32)), host(np.zeros(b.result_entries, np.float32)))
    gi, gd = b.run_host(hc, hq, out=out)
    H.assert_identical(gi[:, None], gd[:, None], di[:, None], dd[:, None], "host run vs device run")
    for c in range(len(clouds)):
        if queries[c].shape[0] == 0:
            assert b.split(gi)[c].size == 0
            continue
        if split_rule == 0:
            oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        else:
            oi, od, _ = O.bf_knn(clouds[c], queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(b.split(gi)[c], b.split(gd)[c], oi, od, f"cloud {c} k={ks[c]} rule {split_rule}")
    del hold
