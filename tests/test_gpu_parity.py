"""GPU parity: the CUDA kd-tree build, kd-tree search and brute force,
called through the C ABI, against the CPU oracle on the same inputs.

Bar: the device tree is the oracle's tree node for node (same cut
dimensions, cut values, children and bucket order); search results are
bit-identical to the oracle's canonical mode (indices, dists2 and the
TOUCH_STATISTICS count), which itself matches the reference's
semantics up to exact distance ties (tests/test_oracle.py).
"""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def _tree_equal(gpu, orc, label):
    g = gpu.export_tree()
    o = orc.export()
    assert gpu.nodeCount == orc.node_count, f"{label}: node count {gpu.nodeCount} vs {orc.node_count}"
    assert gpu.height == orc.height, f"{label}: height {gpu.height} vs {orc.height}"
    for key in ("cut_dim", "right", "bucket_start", "bucket_count", "buckets"):
        bad = np.nonzero(g[key] != o[key])[0]
        assert bad.size == 0, f"{label}: {key} differs at {bad[:5]}: {g[key][bad[:5]]} vs {o[key][bad[:5]]}"
    inner = o["cut_dim"] >= 0
    assert (g["cut_val"][inner] == o["cut_val"][inner]).all(), f"{label}: cut values differ"


def _clouds():
    rng = np.random.default_rng(42)
    grid = np.stack(np.meshgrid(np.arange(9), np.arange(9), np.arange(9), indexing="ij"), -1).reshape(-1, 3)
    yield "uniform3", rng.random((20000, 3)).astype(np.float32)
    yield "uniform3_f64", rng.random((7000, 3))
    yield "grid_dups", np.concatenate([grid, grid[::3]]).astype(np.float32)
    yield "all_equal", np.full((300, 3), 0.25, np.float32)
    yield "negative", (-5.0 - rng.random((3000, 3))).astype(np.float32)
    yield "skewed", (rng.random((5000, 2)) ** 8).astype(np.float32)
    yield "tiny", rng.random((5, 3)).astype(np.float32)
    yield "one_point", np.array([[1.0, 2.0, 3.0]], np.float32)
    yield "lidar_small", __import__("libnabo_gb300.synthetic", fromlist=["x"]).lidar_scan(n_azimuth=600)


@pytest.mark.parametrize("bucket", [2, 3, 8, 17])
def test_tree_identical_to_oracle(bucket):
    nb = _nb()
    for name, cloud in _clouds():
        gpu = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params={"bucketSize": bucket})
        orc = O.OracleTree(cloud, bucket_size=bucket)
        _tree_equal(gpu, orc, f"{name}/B{bucket}")
        o = orc.export()
        assert np.array_equal(gpu.minBound, o["min_bound"]) and np.array_equal(gpu.maxBound, o["max_bound"])


def test_tree_identical_to_oracle_many_small_segments():
    """A cloud of 8 M points: about 40 k small segments, each built by one
    warp, many more than the warps resident at once."""
    nb = _nb()
    cloud = np.random.default_rng(77).random((8_000_000, 3)).astype(np.float32)
    _tree_equal(nb.NearestNeighbourSearch(cloud), O.OracleTree(cloud), "uniform 8M")


@pytest.mark.parametrize("case", H.KNNVALIDATE_CASES, ids=lambda c: f"{c[0]}-m{c[3]}-r{c[4]}")
def test_knnvalidate_cases_gpu(ref_scans, case):
    """tests/knnvalidate.cpp on the reference clouds, with the CUDA types."""
    nb = _nb()
    name, K, dim, method, max_radius = case
    cloud = ref_scans[name].astype(np.float32)
    it_count = method if method != -1 else cloud.shape[0] * 2
    q = H.create_query(cloud, it_count, method)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    _tree_equal(nb.NearestNeighbourSearch(cloud), O.OracleTree(cloud), name)
    ib, db, _ = O.bf_knn(cloud, q, K, H.SORT_RESULTS, max_radius, mode=O.MODE_REFERENCE)
    ic, dc, tc = orc.knn(q, K, 0.0, H.SORT_RESULTS, max_radius, mode=O.MODE_CANONICAL)
    for st in (nb.SearchType.KDTREE_CUDA, nb.SearchType.BRUTE_FORCE_CUDA):
        s = nb.NearestNeighbourSearch(cloud, st, creationOptionFlags=nb.TOUCH_STATISTICS)
        idx, d2 = s.knn(q, K, 0.0, nb.SORT_RESULTS, max_radius)
        H.knnvalidate_check(cloud, q, ib, db, idx, f"{name} {st.name}")
        H.assert_identical(idx, d2, ic, dc, f"{name} {st.name} vs oracle")
        if st == nb.SearchType.KDTREE_CUDA:
            assert s.touched == tc
        else:
            assert s.touched == q.shape[0] * cloud.shape[0]


def _check_against_oracle(cloud, q, k, eps=0.0, flags=0, max_radius=np.inf, radii=None, bucket=8):
    """Both kd-tree traversals and brute force against the oracle.

    The default reference-order kernel must match the oracle's kd-tree
    search: indices, dists2 and the touched count. The opt-in warp-packet
    kernel (traversal=2, exact searches) prunes with a bound that provably
    never exceeds a point's distance, so it must match the oracle's brute
    force exactly; the reference's incrementally updated box distance can
    round above a point's distance, so on rare inputs where a point ties the
    head at that rounding the kd-tree search misses a point that brute force
    keeps (see test_empty_query_and_far_queries).
    """
    nb = _nb()
    orc = O.OracleTree(cloud, bucket_size=bucket, creation_flags=H.TOUCH_STATISTICS)
    oi, od, ot = orc.knn(q, k, eps, flags, max_radius, max_radii=radii, mode=O.MODE_CANONICAL)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS,
                                  params={"bucketSize": bucket})
    gi, gd = s.knn(q, k, eps, flags, max_radius, maxRadii=radii)
    H.assert_identical(gi, gd, oi, od, f"kd-tree k={k} eps={eps} flags={flags}")
    assert s.touched == ot, f"touched {s.touched} vs {ot}"
    r = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params={"bucketSize": bucket})
    ri, rd = r.knn(q, k, eps, flags, max_radius, maxRadii=radii)
    H.assert_identical(ri, rd, oi, od, f"kd-tree without statistics k={k} eps={eps} flags={flags}")
    if eps == 0.0:
        bi, bd, _ = O.bf_knn(cloud, q, k, flags, max_radius, max_radii=radii, mode=O.MODE_CANONICAL)
        p = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, params={"bucketSize": bucket, "traversal": 2})
        pi, pd = p.knn(q, k, eps, flags, max_radius, maxRadii=radii)
        H.assert_identical(pi, pd, bi, bd, f"kd-tree (warp packet) vs oracle brute force k={k}")
        H.assert_equal_up_to_ties(pi, pd, oi, od, f"kd-tree (warp packet) vs oracle kd-tree k={k}")
        b = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA)
        gbi, gbd = b.knn(q, k, 0.0, flags, max_radius, maxRadii=radii)
        H.assert_identical(gbi, gbd, bi, bd, f"brute force k={k}")
    return gi, gd


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [2, 3, 4, 5, 8, 16])
def test_dims_and_types(dtype, d):
    rng = np.random.default_rng(100 + d)
    cloud = rng.random((4000, d)).astype(dtype)
    q = rng.random((1500, d)).astype(dtype)
    for k in (1, 7, 10):
        _check_against_oracle(cloud, q, k)


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 9, 10, 16, 24, 32])
def test_k_values(k):
    rng = np.random.default_rng(k)
    cloud = rng.random((6000, 3)).astype(np.float32)
    q = rng.random((3000, 3)).astype(np.float32)
    _check_against_oracle(cloud, q, k, flags=H.SORT_RESULTS)


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_self_match_flags(flags):
    rng = np.random.default_rng(5)
    cloud = rng.random((5000, 3)).astype(np.float32)
    q = np.concatenate([cloud[:2000], rng.random((1000, 3)).astype(np.float32)])
    gi, _ = _check_against_oracle(cloud, q, 6, flags=flags)
    if flags & H.ALLOW_SELF_MATCH:
        assert (gi[:2000, 0] == np.arange(2000)).all()
    else:
        assert (gi[:2000] != np.arange(2000)[:, None]).all()


@pytest.mark.parametrize("eps", [0.1, 0.5, 2.0])
def test_approximate_epsilon(eps):
    rng = np.random.default_rng(11)
    cloud = rng.random((20000, 3)).astype(np.float32)
    q = rng.random((5000, 3)).astype(np.float32)
    gi, gd = _check_against_oracle(cloud, q, 10, eps=eps)
    # (1+eps) bound against the exact search
    ei, ed, _ = O.bf_knn(cloud, q, 10, mode=O.MODE_CANONICAL)
    bound = (np.float32(1 + eps) ** 2) * ed
    assert (gd <= bound * (1 + 1e-6)).all()


def test_radius_and_per_query_radii():
    rng = np.random.default_rng(12)
    cloud = rng.random((20000, 3)).astype(np.float32)
    q = rng.random((4000, 3)).astype(np.float32)
    _check_against_oracle(cloud, q, 10, max_radius=0.04)
    radii = rng.uniform(0.0, 0.08, 4000).astype(np.float32)
    gi, gd = _check_against_oracle(cloud, q, 10, radii=radii)
    assert ((gi < 0) == np.isinf(gd)).all() and (gi < 0).any()


def test_degenerate_clouds():
    nb = _nb()
    for name, cloud in _clouds():
        n = cloud.shape[0]
        q = np.concatenate([cloud[: min(n, 500)], cloud[: min(n, 500)] + 0.01]).astype(cloud.dtype)
        k = max(1, min(10, n - 1))
        if n > 1:
            _check_against_oracle(cloud, q, k)
        _check_against_oracle(cloud, q, min(10, n), flags=H.ALLOW_SELF_MATCH)


def test_empty_query_and_far_queries():
    """Queries 1e7 away from a unit cloud: every squared distance rounds to
    one of a few float values, so most neighbours tie. The brute-force and
    warp-packet answers keep the lowest indices among the tied points; the
    reference-order traversal can prune a cell whose incrementally updated
    box distance rounded above the head while a point inside it ties the
    head, which the oracle's kd-tree reproduces."""
    nb = _nb()
    rng = np.random.default_rng(13)
    cloud = rng.random((1000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    idx, d2 = s.knn(np.zeros((0, 3), np.float32), 4)
    assert idx.shape == (0, 4)
    far = rng.random((100, 3)).astype(np.float32) * 1e6 + 1e7
    _check_against_oracle(cloud, far, 4)


def test_double_far_queries_ties_and_nan_radii():
    """Double clouds: exact searches decide the reference's traversal on
    float bounds and fall back to the double traversal when a decision is not
    certain. Queries 1e16 away from a unit cloud make every squared distance
    round to a few double values (ties at the head, cells whose rounded box
    distance sits on the head), and NaN radii pass nothing: results and
    touched counts must still be the oracle kd-tree's."""
    rng = np.random.default_rng(31)
    cloud = rng.random((2000, 3))
    far = rng.random((300, 3)) * 1e15 + 1e16
    _check_against_oracle(cloud, far, 4)
    _check_against_oracle(cloud, far, 16)
    q = rng.random((400, 3))
    radii = rng.uniform(0.01, 0.2, 400)
    radii[::7] = np.nan
    _check_against_oracle(cloud, q, 6, radii=radii)
    grid = np.stack(np.meshgrid(*[np.arange(7.0)] * 3, indexing="ij"), -1).reshape(-1, 3)
    _check_against_oracle(grid, grid[::5] + 0.5, 8)


def test_search_errors_match_reference_messages():
    nb = _nb()
    rng = np.random.default_rng(14)
    cloud = rng.random((10, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    orc = O.OracleTree(cloud)
    cases = [dict(k=10), dict(k=11, optionFlags=1), dict(k=2, optionFlags=4)]
    for c in cases:
        with pytest.raises(nb.NaboError) as eg:
            s.knn(cloud, c["k"], 0.0, c.get("optionFlags", 0))
        with pytest.raises(O.OracleError) as eo:
            orc.knn(cloud, c["k"], 0.0, c.get("optionFlags", 0))
        assert str(eg.value) == str(eo.value)
    with pytest.raises(nb.NaboError, match="Query has less dimensions"):
        s.knn(cloud[:, :2], 2)
    with pytest.raises(nb.NaboError, match="k larger than 1024"):
        nb.NearestNeighbourSearch(rng.random((2000, 3)).astype(np.float32)).knn(cloud, 1025)


def test_device_api_matches_host_api():
    import torch
    nb = _nb()
    rng = np.random.default_rng(15)
    cloud = rng.random((30000, 3)).astype(np.float32)
    q = rng.random((20000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    hi, hd = s.knn(q, 10)
    ht = s.touched
    tq = torch.from_numpy(q).cuda()
    touched = torch.zeros(1, dtype=torch.int64, device="cuda")
    di, dd = s.knn_device(tq, 10, touched=touched)
    torch.cuda.synchronize()
    H.assert_identical(di.cpu().numpy(), dd.cpu().numpy(), hi, hd, "device vs host")
    assert int(touched.item()) == ht
    # a cloud given as a CUDA tensor builds the same tree
    s2 = nb.NearestNeighbourSearch(torch.from_numpy(cloud).cuda())
    _tree_equal(s2, O.OracleTree(cloud), "device cloud")


def test_query_ordering_does_not_change_results():
    nb = _nb()
    rng = np.random.default_rng(16)
    cloud = rng.random((50000, 3)).astype(np.float32)
    q = rng.random((30000, 3)).astype(np.float32)
    a = nb.NearestNeighbourSearch(cloud, params={"queryOrdering": 1})
    b = nb.NearestNeighbourSearch(cloud, params={"queryOrdering": 0})
    ia, da = a.knn(q, 10)
    ib, db = b.knn(q, 10)
    H.assert_identical(ia, da, ib, db, "ordering")


def test_uniform_10k_config():
    """10,000 uniform points, 10,000 queries, k=5, eps=0, bucketSize=8,
    SORT_RESULTS: kd-tree and brute force identical, both equal to the oracle."""
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    cloud = S.uniform(10000, 3, seed=S.SEED_BASE)
    q = S.uniform(10000, 3, seed=S.SEED_BASE + 100)
    t = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA)
    b = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA)
    ti, td = t.knn(q, 5, 0.0, nb.SORT_RESULTS)
    bi, bd = b.knn(q, 5, 0.0, nb.SORT_RESULTS)
    H.assert_identical(ti, td, bi, bd, "tree vs bf")
    oi, od, _ = O.bf_knn(cloud, q, 5, H.SORT_RESULTS, mode=O.MODE_CANONICAL)
    H.assert_identical(ti, td, oi, od, "tree vs oracle")
    np.testing.assert_allclose(td, od, rtol=1e-6)


@pytest.mark.parametrize("which", ["lidar", "uniform"])
def test_full_size_properties(which):
    """Full-size clouds (about 1.15M lidar returns / 1M uniform points): size-
    independent properties on every query, exact oracle agreement on a sample."""
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    if which == "lidar":
        cloud = S.lidar_scan()
        q = S.lidar_queries(cloud)
        k, r, flags = 10, 1.0, 0
    else:
        cloud = S.uniform(1_000_000, 3, seed=S.SEED_BASE + 5)
        q = S.uniform(1_000_000, 3, seed=S.SEED_BASE + 6)
        k, r, flags = 10, np.inf, 0
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud)
    _tree_equal(s, orc, which)
    gi, gd = s.knn(q, k, 0.0, flags, r)
    rows = np.random.default_rng(0).choice(q.shape[0], 2000, replace=False)
    H.check_sorted_and_consistent(cloud, q[rows], gi[rows], gd[rows], k)
    sample = np.random.default_rng(1).choice(q.shape[0], 20000, replace=False)
    oi, od, _ = orc.knn(q[sample], k, 0.0, flags, r, mode=O.MODE_CANONICAL)
    H.assert_identical(gi[sample], gd[sample], oi, od, f"{which} sample")
    # without statistics, and with the warp-packet traversal, every query
    # gets the same answer
    for params in ({}, {"traversal": 2}):
        p = nb.NearestNeighbourSearch(cloud, params=params)
        pi, pd = p.knn(q, k, 0.0, flags, r)
        H.assert_identical(pi, pd, gi, gd, f"{which} {params} vs statistics run")


def test_non_finite_cloud_is_rejected():
    nb = _nb()
    cloud = np.random.default_rng(3).random((500, 3)).astype(np.float32)
    for bad in (np.nan, np.inf, -np.inf):
        c = cloud.copy()
        c[123, 1] = bad
        with pytest.raises(nb.NaboError, match="non-finite"):
            nb.NearestNeighbourSearch(c)
    # a non-finite value in a row beyond `dim` is not searched and is accepted
    c = np.concatenate([cloud, np.full((500, 1), np.nan, np.float32)], axis=1)
    s = nb.NearestNeighbourSearch(c, dim=3)
    assert s.dim == 3


@pytest.mark.parametrize("case", ["huge", "tiny", "offset", "far_queries", "mixed_scale"])
def test_double_prefilter_edge_cases(case):
    """Double clouds are searched with a float pre-filter of leaf points (a
    float lower bound of each squared distance with a proven margin). Its
    edge cases must still give the oracle's exact answer: coordinates beyond
    the float range (the margin becomes infinite), values that are subnormal
    or zero in float, a large common offset with tiny separations (float
    cancellation), queries far from the cloud, and mixed scales."""
    rng = np.random.default_rng(["huge", "tiny", "offset", "far_queries", "mixed_scale"].index(case) + 500)
    if case == "huge":
        cloud = rng.random((3000, 3)) * 1e40
        q = rng.random((800, 3)) * 1e40
    elif case == "tiny":
        cloud = rng.random((3000, 3)) * 1e-40
        q = rng.random((800, 3)) * 1e-40
    elif case == "offset":
        cloud = 1e6 + rng.random((3000, 3)) * 1e-3
        q = 1e6 + rng.random((800, 3)) * 1e-3
    elif case == "far_queries":
        cloud = rng.random((3000, 3))
        q = rng.random((800, 3)) * 1e3 + 1e5
    else:
        cloud = np.concatenate([rng.random((1500, 3)) * 1e-6, rng.random((1500, 3)) * 1e6])
        q = np.concatenate([rng.random((400, 3)) * 1e-6, rng.random((400, 3)) * 1e6])
    for k in (1, 10, 32):
        _check_against_oracle(cloud.astype(np.float64), q.astype(np.float64), k)
