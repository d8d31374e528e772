"""The median-split tree (splitRule 1): a balanced kd-tree with the search's
node layout, the alternate layout the batched autotuner may choose (the
balanced trees of nabo/kdtree_opencl.cpp:474-514, with buckets). It is not
the reference's tree, so results are checked against the oracle's brute
force (the exact k smallest (dist2, index) pairs), and TOUCH_STATISTICS,
which would not count what the reference counts, is refused."""
import math

import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def _clouds():
    from libnabo_gb300 import synthetic as S
    lidar = S.lidar_scan(n_azimuth=2400)
    c8, _, _ = S.clusters(30000, 8, 5, dtype=np.float64)
    return {
        "uniform_f32": (S.uniform(50000, 3, seed=3), S.uniform(8000, 3, seed=4)),
        "lidar_f32": (lidar, S.lidar_queries(lidar)[:8000]),
        "clusters8_f64": (c8, (c8[:6000] + np.random.default_rng(6).normal(0, 0.01, (6000, 8))).astype(np.float64)),
    }


@pytest.mark.parametrize("name", ["uniform_f32", "lidar_f32", "clusters8_f64"])
@pytest.mark.parametrize("k", [1, 10, 40])
def test_median_tree_search_is_exact(name, k):
    nb = _nb()
    cloud, q = _clouds()[name]
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params={"splitRule": 1})
    # balanced: splits near the median (sampled at the level-synchronous
    # levels, ties to the left), so the height stays within a few levels of
    # log2(n / bucket)
    assert tree.height <= math.ceil(math.log2(cloud.shape[0] / 8)) + 4, tree.height
    for opt in (0, nb.ALLOW_SELF_MATCH):
        gi, gd = tree.knn(q, k, 0.0, opt)
        oi, od, _ = O.bf_knn(cloud, q, k, opt, mode=O.MODE_CANONICAL)
        H.assert_identical(gi, gd, oi, od, f"{name} k={k} opt={opt}")
    gi, gd = tree.knn(q, k, 0.0, 0, 0.05)
    oi, od, _ = O.bf_knn(cloud, q, k, 0, 0.05, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"{name} k={k} radius")


def test_median_tree_refuses_touch_statistics():
    nb = _nb()
    cloud = np.random.default_rng(0).random((1000, 3)).astype(np.float32)
    with pytest.raises(nb.NaboError) as e:
        nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS,
                                  params={"splitRule": 1})
    assert e.value.code == 1 and "TOUCH_STATISTICS" in str(e.value)


@pytest.mark.parametrize("graph", [False, True])
def test_median_tree_batches_are_exact(graph):
    import torch
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    sizes = S.log_uniform_sizes(24, 300, 40000, 9)
    rng = np.random.default_rng(10)
    clouds = [S.gaussian_blobs(int(n), 30 + i) for i, n in enumerate(sizes)]
    queries = [(c + rng.normal(0, 0.01, c.shape)).astype(np.float32) for c in clouds]
    ks = np.minimum(rng.choice([1, 5, 16], len(clouds)), sizes - 1).astype(np.int32)
    b = nb.BatchSearch([c.shape[0] for c in clouds], splitRule=1, maxLevels=40)
    b.set_queries([q.shape[0] for q in queries], ks)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    if graph:
        idx, d2 = b.run(tc, tq)
    else:
        b.build(tc)
        idx, d2 = b.knn(tq)
    torch.cuda.synchronize()
    assert b.status()["ok"], b.status()
    bi, bd = b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())
    for c in range(0, len(clouds), 3):
        oi, od, _ = O.bf_knn(clouds[c], queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(bi[c], bd[c], oi, od, f"median-split batch cloud {c}")
