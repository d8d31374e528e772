"""kd-trees of any height, against the oracle.

The reference's recursion (nabo/kdtree_cpu.cpp:367-447) has no depth limit,
and its sliding-midpoint split gives a tree as tall as the cloud is large on
geometrically spaced coordinates: on points (2^i, 0, 0), (0, 2^i, 0) and
(0, 0, 2^i) each split peels off about one point. The search kernels keep
256 levels of stack in local memory; taller trees search with their stacks
in global memory (one query per thread for k <= 32, a lane group per query
above), and batches hand the queries of taller trees to that search from
inside the same launch sequence. Results must be bit-identical to the
oracle's canonical mode, TOUCH_STATISTICS included.
"""
import ctypes

import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def axis_geometric(dtype, lo, hi, dims=3):
    """Points 2^i on each axis, i in [lo, hi): a tree of height ~ N."""
    exps = np.arange(lo, hi, dtype=np.float64)
    pts = np.zeros((dims * exps.size, dims), np.float64)
    for d in range(dims):
        pts[d * exps.size:(d + 1) * exps.size, d] = 2.0 ** exps
    return pts.astype(dtype)


def tall_queries(cloud, n, seed):
    """Points near the cloud's axes at every scale, the cloud's own points,
    and points between the axes."""
    rng = np.random.default_rng(seed)
    dims = cloud.shape[1]
    m = n // 3
    src = cloud[rng.integers(0, cloud.shape[0], m)].astype(np.float64)
    near = src * (1.0 + rng.normal(0, 0.3, src.shape)) + rng.normal(0, 1e-3, src.shape) * np.abs(src).max(1, keepdims=True)
    own = cloud[rng.integers(0, cloud.shape[0], m)].astype(np.float64)
    mag = 2.0 ** rng.uniform(-40, 20, (n - 2 * m, 1))
    between = rng.uniform(-1, 1, (n - 2 * m, dims)) * mag
    return np.concatenate([near, own, between]).astype(cloud.dtype)


CLOUDS = {
    "f32": (np.float32, -100, 64),   # 492 points, height 481
    "f64": (np.float64, -600, 512),  # 3336 points, height 3325
}


@pytest.fixture(scope="module", params=sorted(CLOUDS))
def tall(request):
    dtype, lo, hi = CLOUDS[request.param]
    cloud = axis_geometric(dtype, lo, hi)
    orc = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)
    assert orc.height > 256
    return request.param, cloud, orc


@pytest.mark.parametrize("k", [1, 10, 64])
@pytest.mark.parametrize("stats", [False, True])
def test_tall_tree_search_matches_oracle(tall, k, stats):
    nb = _nb()
    name, cloud, orc = tall
    q = tall_queries(cloud, 3000, seed=11)
    flags = nb.TOUCH_STATISTICS if stats else 0
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=flags)
    assert tree.height == orc.height
    for opt in (0, nb.ALLOW_SELF_MATCH):
        gi, gd = tree.knn(q, k, 0.0, opt | nb.SORT_RESULTS)
        oi, od, ot = orc.knn(q, k, 0.0, opt | O.SORT_RESULTS, mode=O.MODE_CANONICAL)
        H.assert_identical(gi, gd, oi, od, f"{name} k={k} opt={opt}")
        if stats:
            assert tree.touched == ot, (tree.touched, ot)


def test_tall_tree_radii_and_epsilon(tall):
    nb = _nb()
    name, cloud, orc = tall
    q = tall_queries(cloud, 2000, seed=12)
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    rng = np.random.default_rng(5)
    radii = (2.0 ** rng.uniform(-30, 10, q.shape[0])).astype(cloud.dtype)
    gi, gd = tree.knn(q, 5, 0.0, 0, maxRadii=radii)
    oi, od, ot = orc.knn(q, 5, 0.0, 0, max_radii=radii, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"{name} per-query radii")
    assert tree.touched == ot
    gi, gd = tree.knn(q, 8, 0.5, 0, 2.0 ** -10)
    oi, od, ot = orc.knn(q, 8, 0.5, 0, 2.0 ** -10, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"{name} eps=0.5, scalar radius")
    assert tree.touched == ot


def test_tall_tree_many_queries_share_the_stacks():
    """More queries than the deep search's stacks can serve at once (each
    thread then searches several queries in turn)."""
    nb = _nb()
    cloud = axis_geometric(np.float64, -1074, 512)  # height 4747
    orc = O.OracleTree(cloud)
    q = tall_queries(cloud, 60000, seed=13)
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA)
    gi, gd = tree.knn(q, 4, 0.0, 0)
    oi, od, _ = orc.knn(q, 4, 0.0, 0, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, "f64 height 4747, 60k queries")


def test_tall_tree_no_alloc_entry_point(tall):
    """The allocation-free entry point searches tall trees with their stacks
    in its fixed array."""
    import torch
    nb = _nb()
    from libnabo_gb300 import _native
    lib = _native.lib
    name, cloud, orc = tall
    q = tall_queries(cloud, 1500, seed=14)
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    tq = torch.from_numpy(q).cuda()
    k = 7
    idx = torch.full((q.shape[0], k), -7, dtype=torch.int32, device="cuda")
    d2 = torch.full((q.shape[0], k), -7.0, dtype=tq.dtype, device="cuda")
    touched = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.nabo_cuda_knn_device_noalloc(tree._h, ctypes.c_void_p(tq.data_ptr()), 3, q.shape[0], 3, k, 0.0, 0,
                                          float("inf"), None, ctypes.c_void_p(idx.data_ptr()),
                                          ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(touched.data_ptr()),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.nabo_cuda_last_error().decode()
    torch.cuda.synchronize()
    oi, od, ot = orc.knn(q, k, 0.0, 0, mode=O.MODE_CANONICAL)
    H.assert_identical(idx.cpu().numpy(), d2.cpu().numpy(), oi, od, f"{name} no-alloc")
    assert int(touched.item()) == ot


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("kind", ["f32", "f64", "f32-wide"])
def test_batch_with_tall_trees(graph, kind):
    """A batch holding tall trees among ordinary clouds: the build reports
    them (status bit 4), every query still gets the oracle's answer."""
    import torch
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    dtype = np.float64 if kind == "f64" else np.float32
    lo, hi = (-300, 100) if kind == "f64" else (-100, 64)
    tall_cloud = axis_geometric(dtype, lo, hi)
    clouds = [S.gaussian_blobs(3000, 21, dtype=dtype), tall_cloud, S.gaussian_blobs(700, 22, dtype=dtype),
              axis_geometric(dtype, lo + 20, hi - 10)]
    queries = [tall_queries(c, 900 + 100 * i, seed=30 + i) for i, c in enumerate(clouds)]
    ks = np.array([40, 33, 64, 50] if kind == "f32-wide" else [5, 16, 1, 10], np.int32)
    levels = max(O.OracleTree(c).height for c in clouds) + 8
    b = nb.BatchSearch([c.shape[0] for c in clouds], dim=3, dtype=dtype, maxLevels=levels)
    b.set_queries([q.shape[0] for q in queries], ks)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    for rep in range(2):  # a second run reuses the overflow list and the graph
        if graph:
            idx, d2 = b.run(tc, tq)
        else:
            b.build(tc)
            idx, d2 = b.knn(tq)
        torch.cuda.synchronize()
        st = b.status()
        assert st["flags"] == 4 and st["ok"], st
        assert st["height"] == max(O.OracleTree(c).height for c in clouds)
        bi, bd = b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())
        for c in range(len(clouds)):
            oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
            H.assert_identical(bi[c], bd[c], oi, od, f"{kind} cloud {c} rep {rep}")
