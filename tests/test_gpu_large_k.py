"""k above 32 (one warp per query, up to k = 1024): the reference's heaps
have no cap on k (nabo/index_heap.h:51-165, 263-369). Kd-tree, brute force
and batched searches against the oracle's canonical mode, bit for bit,
with the radius, epsilon, self-match and per-query-radius variants of the
reference's knn (nabo/kdtree_cpu.cpp:274-336) and the TOUCH_STATISTICS
count."""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def _data(n, nq, dim, dtype, seed):
    rng = np.random.default_rng(seed)
    cloud = rng.random((n, dim)).astype(dtype)
    # half the queries are cloud points (self matches, exact ties), half free
    q = np.concatenate([cloud[rng.choice(n, nq // 2, replace=False)], rng.random((nq - nq // 2, dim))]).astype(dtype)
    return cloud, q


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("dim", [2, 3, 8])
@pytest.mark.parametrize("k", [33, 64, 100, 257, 1024])
def test_kdtree_large_k_matches_oracle(dtype, dim, k):
    nb = _nb()
    cloud, q = _data(6000 if k < 1024 else 3000, 700, dim, dtype, seed=100 + dim + k)
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    r = 0.12 if dim <= 3 else 0.6
    cases = [dict(), dict(maxRadius=r), dict(epsilon=0.5), dict(optionFlags=H.ALLOW_SELF_MATCH),
             dict(epsilon=0.25, maxRadius=r, optionFlags=H.ALLOW_SELF_MATCH | H.SORT_RESULTS)]
    for c in cases:
        idx, d2 = s.knn(q, k, c.get("epsilon", 0.0), c.get("optionFlags", 0), c.get("maxRadius", np.inf))
        oi, od, ot = orc.knn(q, k, c.get("epsilon", 0.0), c.get("optionFlags", 0), c.get("maxRadius", np.inf),
                             mode=O.MODE_CANONICAL)
        H.assert_identical(idx, d2, oi, od, f"k={k} dim={dim} {c}")
        assert s.touched == ot, (c, s.touched, ot)
    radii = np.random.default_rng(k).uniform(0.02, 2 * r, q.shape[0]).astype(dtype)
    idx, d2 = s.knn(q, k, maxRadii=radii)
    oi, od, ot = orc.knn(q, k, max_radii=radii, mode=O.MODE_CANONICAL)
    H.assert_identical(idx, d2, oi, od, f"k={k} dim={dim} per-query radii")
    assert s.touched == ot


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("k", [33, 200, 1024])
def test_bruteforce_large_k_matches_oracle(dtype, k):
    nb = _nb()
    cloud, q = _data(5000, 300, 3, dtype, seed=7 + k)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA)
    for c in (dict(), dict(maxRadius=0.1), dict(optionFlags=H.ALLOW_SELF_MATCH)):
        idx, d2 = s.knn(q, k, 0.0, c.get("optionFlags", 0), c.get("maxRadius", np.inf))
        oi, od, _ = O.bf_knn(cloud, q, k, c.get("optionFlags", 0), c.get("maxRadius", np.inf),
                             mode=O.MODE_CANONICAL)
        H.assert_identical(idx, d2, oi, od, f"bf k={k} {c}")


def test_large_k_whole_cloud_and_ties():
    """k = n - 1 returns every other point; a grid with many equal distances
    keeps the (dist2, index) order."""
    nb = _nb()
    g = np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij"), -1).reshape(-1, 3)
    cloud = g.astype(np.float32)
    n = cloud.shape[0]
    for st in (nb.SearchType.KDTREE_CUDA, nb.SearchType.BRUTE_FORCE_CUDA):
        s = nb.NearestNeighbourSearch(cloud, st)
        for k in (n - 1, 100, 40):
            idx, d2 = s.knn(cloud, k)
            oi, od, _ = O.bf_knn(cloud, cloud, k, mode=O.MODE_CANONICAL)
            H.assert_identical(idx, d2, oi, od, f"{st.name} grid k={k}")
        idx, _ = s.knn(cloud, n - 1)
        for i in range(0, n, 37):
            assert sorted(idx[i].tolist()) == [j for j in range(n) if j != i]


def test_large_k_limits():
    nb = _nb()
    rng = np.random.default_rng(5)
    cloud = rng.random((3000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    with pytest.raises(nb.NaboError, match="k larger than 1024"):
        s.knn(cloud[:10], 1025)
    # the warp-packet traversal serves k <= 32; larger k take the warp-per-query search
    s2 = nb.NearestNeighbourSearch(cloud, params={"traversal": 2})
    idx, d2 = s2.knn(cloud[:500], 50)
    oi, od, _ = O.OracleTree(cloud).knn(cloud[:500], 50, mode=O.MODE_CANONICAL)
    H.assert_identical(idx, d2, oi, od, "packet flag, k=50")


def test_device_api_large_k():
    import torch
    nb = _nb()
    cloud, q = _data(20000, 5000, 3, np.float32, seed=77)
    s = nb.NearestNeighbourSearch(cloud)
    di, dd = s.knn_device(torch.from_numpy(q).cuda(), 48)
    torch.cuda.synchronize()
    oi, od, _ = O.OracleTree(cloud).knn(q, 48, mode=O.MODE_CANONICAL)
    H.assert_identical(di.cpu().numpy(), dd.cpu().numpy(), oi, od, "device api k=48")


def test_batch_with_large_k_cloud():
    import torch
    from libnabo_gb300 import synthetic as S
    nb = _nb()
    sizes = [400, 3000, 9000, 70]
    clouds = [S.gaussian_blobs(n, 500 + i) for i, n in enumerate(sizes)]
    rng = np.random.default_rng(9)
    queries = [(c + rng.normal(0, 0.01, c.shape)).astype(np.float32) for c in clouds]
    ks = np.array([40, 5, 130, 69], np.int32)
    b = nb.BatchSearch(sizes, dim=3)
    b.set_queries([x.shape[0] for x in queries], ks)
    b.build(torch.from_numpy(np.concatenate(clouds)).cuda())
    idx, d2 = b.knn(torch.from_numpy(np.concatenate(queries)).cuda())
    torch.cuda.synchronize()
    gi, gd = b.split(idx.cpu().numpy()), b.split(d2.cpu().numpy())
    for c in range(len(sizes)):
        oi, od, _ = O.OracleTree(clouds[c]).knn(queries[c], int(ks[c]), mode=O.MODE_CANONICAL)
        H.assert_identical(gi[c], gd[c], oi, od, f"batch cloud {c} k={ks[c]}")


def test_learned_radius_large_k():
    """The learned-radius search with k above 32: bounded searches that miss
    rerun without the bound inside the warp, so results equal the plain
    search's."""
    nb = _nb()
    cloud, q = _data(30000, 20000, 3, np.float32, seed=31)
    s = nb.NearestNeighbourSearch(cloud)
    m = nb.RadiusModel(s, q[:8000], k=40, epochs=4)
    pi, pd = s.knn(q, 40)
    li, ld = m.knn(q, 40)
    H.assert_identical(li, ld, pi, pd, "learned k=40")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("dim,bucket", [(16, 8), (3, 17), (8, 33)])
def test_large_k_wide_records_and_big_buckets(dtype, dim, bucket):
    """16-dimensional records (the groups' stacks outgrow the default shared
    memory) and buckets larger than a lane group (a leaf takes several
    passes of the group)."""
    nb = _nb()
    cloud, q = _data(8000, 600, dim, dtype, seed=dim * 100 + bucket)
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS, params={"bucketSize": bucket})
    orc = O.OracleTree(cloud, bucket_size=bucket, creation_flags=H.TOUCH_STATISTICS)
    for k in (40, 128, 300):
        idx, d2 = s.knn(q, k)
        oi, od, ot = orc.knn(q, k, mode=O.MODE_CANONICAL)
        H.assert_identical(idx, d2, oi, od, f"dim={dim} bucket={bucket} k={k}")
        assert s.touched == ot


def test_large_k_tall_tree_smaller_blocks():
    """A double 16-D tree about 110 levels tall: the lane groups' stacks
    need more shared memory than a block may have, so blocks shrink."""
    nb = _nb()
    rng = np.random.default_rng(3)
    n = 800
    cloud = rng.random((n, 16)) * 1e-30
    cloud[:, 0] = 0.5 ** (np.arange(n) / 2)  # crowded along one axis: a deep chain of splits
    q = cloud[rng.choice(n, 300, replace=False)] * (1 + rng.normal(0, 1e-3, (300, 16)))
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    assert orc.height > 100 and s.height == orc.height
    for k in (64, 200):
        idx, d2 = s.knn(q, k)
        oi, od, ot = orc.knn(q, k, mode=O.MODE_CANONICAL)
        H.assert_identical(idx, d2, oi, od, f"tall tree k={k}")
        assert s.touched == ot
