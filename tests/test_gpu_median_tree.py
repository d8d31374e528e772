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
    c16, _, _ = S.clusters(20000, 16, 6, dtype=np.float32)
    return {
        "uniform_f32": (S.uniform(50000, 3, seed=3), S.uniform(8000, 3, seed=4)),
        "lidar_f32": (lidar, S.lidar_queries(lidar)[:8000]),
        "clusters8_f64": (c8, (c8[:6000] + np.random.default_rng(6).normal(0, 0.01, (6000, 8))).astype(np.float64)),
        "uniform4_f32": (S.uniform(40000, 4, seed=7), S.uniform(6000, 4, seed=8)),
        "uniform2_f32": (S.uniform(40000, 2, seed=11), S.uniform(6000, 2, seed=12)),
        "clusters16_f32": (c16, (c16[:5000] + np.random.default_rng(13).normal(0, 0.01, (5000, 16))).astype(np.float32)),
        "uniform3_f64": (S.uniform(40000, 3, seed=9).astype(np.float64), S.uniform(6000, 3, seed=10).astype(np.float64)),
    }


@pytest.mark.parametrize("name", ["uniform_f32", "lidar_f32", "clusters8_f64", "uniform4_f32", "uniform3_f64",
                                  "uniform2_f32", "clusters16_f32"])
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


def _tied_clouds(dtype=np.float32):
    """Clouds that exercise every split choice of the level-synchronous
    levels: few distinct values (ties at the median: the cut at the median
    itself), all points equal (a positional split), one constant
    coordinate, and clouds whose root is already a small segment."""
    from libnabo_gb300 import synthetic as S
    rng = np.random.default_rng(21)
    grid = rng.integers(0, 5, (6000, 3)).astype(dtype)
    same = np.tile(np.array([[0.25, -1.5, 3.0]], dtype), (3000, 1))
    flat = rng.random((5000, 3)).astype(dtype)
    flat[:, 2] = 7.0
    half = np.concatenate([np.zeros((2500, 3)), rng.random((1500, 3))]).astype(dtype)
    return [S.gaussian_blobs(3, 40, dtype=dtype), grid, S.gaussian_blobs(200, 41, dtype=dtype), same,
            S.gaussian_blobs(256, 42, dtype=dtype), flat, half, S.gaussian_blobs(9000, 43, dtype=dtype)]


def _queries_for(clouds, seed):
    rng = np.random.default_rng(seed)
    return [(c[rng.integers(0, c.shape[0], min(c.shape[0], 700))] + rng.normal(0, 0.3, (min(c.shape[0], 700), 3)))
            .astype(c.dtype) for c in clouds]


def assert_valid_tree(t, cloud, bucket, label):
    """A kd-tree whose leaves hold a permutation of the cloud, with every
    point inside its leaf's cell: at or below each ancestor's cut on the
    left side, at or above it on the right (left child = next node)."""
    n = cloud.shape[0]
    order = t["buckets"]
    assert np.array_equal(np.sort(order), np.arange(n)), f"{label}: leaves are not a permutation of the cloud"
    lo = np.full(cloud.shape[1], -np.inf)
    hi = np.full(cloud.shape[1], np.inf)
    stack = [(0, lo, hi)]
    seen = 0
    while stack:
        node, lo, hi = stack.pop()
        d = int(t["cut_dim"][node])
        if d < 0:
            a, c = int(t["bucket_start"][node]), int(t["bucket_count"][node])
            pts = cloud[order[a:a + c]].astype(np.float64)
            assert ((pts >= lo) & (pts <= hi)).all(), f"{label}: leaf {node} holds a point outside its cell"
            assert c <= bucket or np.all(pts == pts[0]), f"{label}: leaf {node} holds {c} points"
            seen += c
            continue
        cut = float(t["cut_val"][node])
        lhi, rlo = hi.copy(), lo.copy()
        lhi[d] = min(hi[d], cut)
        rlo[d] = max(lo[d], cut)
        stack.append((int(t["right"][node]), rlo, hi))
        stack.append((node + 1, lo, lhi))
    assert seen == n, f"{label}: leaves hold {seen} of {n} points"


def assert_exact_up_to_ties(cloud, q, k, gi, gd, label):
    """Squared distances bit-identical to brute force; each returned index
    is a point at its returned distance, none twice. Which of several
    points at exactly the same distance comes back follows the traversal:
    the reference's incremental cell distance (nabo/kdtree_cpu.cpp:415-417, 433-435)
    can round one ulp above a tied point's distance, so its own tree and
    search differ from brute force the same way on such clouds."""
    oi, od, _ = O.bf_knn(cloud, q, k, mode=O.MODE_CANONICAL)
    assert np.array_equal(gd.view(np.uint8), od.view(np.uint8)), f"{label}: distances differ"
    wide = min(cloud.shape[0] - 1, k + 120)
    wi, wd, _ = O.bf_knn(cloud, q, wide, mode=O.MODE_CANONICAL)
    for r in range(q.shape[0]):
        assert len(set(gi[r].tolist())) == k, f"{label}: row {r} repeats an index"
        pairs = set(zip(wi[r].tolist(), wd[r].tolist()))
        assert all((int(i), float(d)) in pairs for i, d in zip(gi[r], gd[r])), f"{label}: row {r}"


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_median_tree_ties_and_duplicates(dtype):
    nb = _nb()
    for i, cloud in enumerate(_tied_clouds(dtype)):
        q = _queries_for([cloud], 50 + i)[0]
        tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params={"splitRule": 1})
        assert_valid_tree(tree.export_tree(), cloud, 8, f"tied cloud {i}")
        k = min(5, cloud.shape[0] - 1)
        gi, gd = tree.knn(q, k, 0.0, 0)
        assert_exact_up_to_ties(cloud, q, k, gi, gd, f"tied cloud {i} {dtype.__name__}")


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("levels", [40, 2])
def test_median_tree_batch_with_ties_small_roots_and_level_limit(graph, levels):
    """The same clouds as one batch. With 2 levels the trees cannot finish:
    the build reports it and every cloud becomes one leaf holding all of its
    points, so results stay exact."""
    import torch
    nb = _nb()
    clouds = _tied_clouds()
    queries = _queries_for(clouds, 60)
    ks = np.array([min(c.shape[0] - 1, k) for c, k in zip(clouds, [1, 5, 16, 4, 16, 5, 10, 16])], np.int32)
    b = nb.BatchSearch([c.shape[0] for c in clouds], splitRule=1, maxLevels=levels)
    b.set_queries([q.shape[0] for q in queries], ks)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    tq = torch.from_numpy(np.concatenate(queries)).cuda()
    for rep in range(2):
        if graph:
            idx, d2 = b.run(tc, tq)
        else:
            b.build(tc)
            idx, d2 = b.knn(tq)
        torch.cuda.synchronize()
        st = b.status()
        if levels == 2:
            assert not st["ok"] and (st["flags"] & 2) and st["nodes"] == len(clouds), st
        else:
            assert st["ok"], st
        bi, bd = b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())
        for c in range(len(clouds)):
            label = f"median batch cloud {c} levels={levels} rep {rep}"
            bucket = clouds[c].shape[0] if levels == 2 else 8
            assert_valid_tree(b.export_tree(c), clouds[c], bucket, label)
            assert_exact_up_to_ties(clouds[c], queries[c], int(ks[c]), bi[c], bd[c], label)


def test_median_tree_batch_8d_is_exact():
    """An 8-D float batch with the median split (the C4 batches' choice for
    float): records of 48 bytes take the unstaged scatter."""
    import torch
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    clouds, queries = [], []
    for i, n in enumerate((2000, 9000, 300, 25000)):
        c, centres, sig = S.clusters(n, 8, 70 + i, dtype=np.float32)
        q, _, _ = S.clusters(700, 8, 90 + i, dtype=np.float32, centres=centres, sigmas=sig)
        clouds.append(c)
        queries.append(q)
    ks = np.array([32, 5, 16, 32], np.int32)
    b = nb.BatchSearch([c.shape[0] for c in clouds], dim=8, splitRule=1, bucketSize=16, maxLevels=40)
    b.set_queries([q.shape[0] for q in queries], ks)
    b.build(torch.from_numpy(np.concatenate(clouds)).cuda())
    idx, d2 = b.knn(torch.from_numpy(np.concatenate(queries)).cuda())
    torch.cuda.synchronize()
    assert b.status()["ok"], b.status()
    bi, bd = b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())
    for c in range(len(clouds)):
        assert_valid_tree(b.export_tree(c), clouds[c], 16, f"8-D median batch cloud {c}")
        oi, od, _ = O.bf_knn(clouds[c], queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(bi[c], bd[c], oi, od, f"8-D median batch cloud {c}")
