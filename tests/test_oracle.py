"""Pins the CPU oracle to the reference's own tests (no GPU needed).

The reference ships no stored outputs; its CTest suite checks the kd-tree
against the in-process brute force on tests/data/*.txt
(tests/knnvalidate.cpp, tests/CMakeLists.txt:9-14) and its usage example
checks self-match behaviour (examples/usage.cpp:32-58). These tests run the
same checks on the oracle, in both its reference mode and the canonical
(lower-index tie) mode the CUDA kernels implement.
"""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

HEAPS = [O.HEAP_LINEAR, O.HEAP_STL]


@pytest.mark.parametrize("case", H.KNNVALIDATE_CASES, ids=lambda c: f"{c[0]}-m{c[3]}-r{c[4]}")
def test_knnvalidate_cases(ref_scans, case):
    name, K, dim, method, max_radius = case
    cloud = ref_scans[name].astype(np.float32)
    assert cloud.shape[1] == dim
    it_count = method if method != -1 else cloud.shape[0] * 2
    q = H.create_query(cloud, it_count, method)
    idx_bf, d2_bf, _ = O.bf_knn(cloud, q, K, H.SORT_RESULTS, max_radius, mode=O.MODE_REFERENCE)
    tree = O.OracleTree(cloud)
    for heap in HEAPS:
        idx, d2, _ = tree.knn(q, K, 0.0, H.SORT_RESULTS, max_radius, mode=O.MODE_REFERENCE, heap=heap)
        H.knnvalidate_check(cloud, q, idx_bf, d2_bf, idx, f"{name} heap={heap}")
    # canonical mode: kd-tree and brute force agree exactly
    idx_c, d2_c, _ = tree.knn(q, K, 0.0, H.SORT_RESULTS, max_radius, mode=O.MODE_CANONICAL)
    idx_cb, d2_cb, _ = O.bf_knn(cloud, q, K, H.SORT_RESULTS, max_radius, mode=O.MODE_CANONICAL)
    H.assert_identical(idx_c, d2_c, idx_cb, d2_cb, f"{name} canonical tree vs bf")
    # canonical and reference modes agree up to exact ties
    idx_r, d2_r, _ = tree.knn(q, K, 0.0, H.SORT_RESULTS, max_radius, mode=O.MODE_REFERENCE)
    H.assert_equal_up_to_ties(idx_c, d2_c, idx_r, d2_r, f"{name} canonical vs reference")


def test_touch_statistics_modes_agree(ref_scans):
    cloud = ref_scans["scan_3d_large"].astype(np.float32)
    q = H.create_query(cloud, 5000, 5000, seed=3)
    tree = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    _, _, t_ref = tree.knn(q, 10, mode=O.MODE_REFERENCE)
    _, _, t_stl = tree.knn(q, 10, mode=O.MODE_REFERENCE, heap=O.HEAP_STL)
    _, _, t_can = tree.knn(q, 10, mode=O.MODE_CANONICAL)
    assert t_ref == t_stl == t_can > 0
    tree0 = O.OracleTree(cloud)
    _, _, t0 = tree0.knn(q, 10)
    assert t0 == 0  # TOUCH_STATISTICS off -> 0 (nabo/nabo.h:323)


def test_self_match_kat():
    """examples/usage.cpp:32-58."""
    rng = np.random.default_rng(7)
    M = rng.uniform(-1, 1, (100, 3)).astype(np.float32)
    tree = O.OracleTree(M)
    idx, _, _ = tree.knn(M, 3, 0.0, H.SORT_RESULTS | H.ALLOW_SELF_MATCH, mode=O.MODE_REFERENCE)
    assert (idx[:, 0] == np.arange(100)).all()
    idx2, _, _ = tree.knn(M, 2, 0.1, 0, mode=O.MODE_REFERENCE)
    assert (idx2[:, 0] != np.arange(100)).all()


def test_unfound_slots_are_padded():
    rng = np.random.default_rng(8)
    cloud = rng.random((2000, 3)).astype(np.float32)
    q = rng.random((300, 3)).astype(np.float32)
    tree = O.OracleTree(cloud)
    for mode in (O.MODE_REFERENCE, O.MODE_CANONICAL):
        idx, d2, _ = tree.knn(q, 16, 0.0, H.SORT_RESULTS, 0.03, mode=mode)
        miss = idx < 0
        assert miss.any() and (~miss).any()
        assert np.isinf(d2[miss]).all() and np.isfinite(d2[~miss]).all()
        assert (d2[~miss] <= np.float32(0.03) * np.float32(0.03)).all()


def test_per_query_radii_match_scalar_radius():
    rng = np.random.default_rng(9)
    cloud = rng.random((5000, 3)).astype(np.float32)
    q = rng.random((1000, 3)).astype(np.float32)
    tree = O.OracleTree(cloud)
    i1, d1, _ = tree.knn(q, 8, max_radius=0.05)
    i2, d2, _ = tree.knn(q, 8, max_radii=np.full(1000, 0.05, np.float32))
    H.assert_identical(i1, d1, i2, d2)


def test_bruteforce_touch_count():
    rng = np.random.default_rng(10)
    cloud = rng.random((700, 3))
    q = rng.random((50, 3))
    _, _, t = O.bf_knn(cloud, q, 4, creation_flags=H.TOUCH_STATISTICS)
    assert t == 700 * 50  # nabo/brute_force_cpu.cpp:99-100


def test_ties_broken_by_lower_index_in_canonical_mode():
    # A grid with many equal distances: canonical tree and brute force agree
    # exactly; the reference-mode tree agrees up to tie choice.
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij"), -1).reshape(-1, 3)
    cloud = g.astype(np.float64)
    q = cloud[::7] + 0.5
    tree = O.OracleTree(cloud, bucket_size=4)
    ic, dc, _ = tree.knn(q, 10, mode=O.MODE_CANONICAL)
    ib, db, _ = O.bf_knn(cloud, q, 10, mode=O.MODE_CANONICAL)
    H.assert_identical(ic, dc, ib, db, "grid canonical")
    ir, dr, _ = tree.knn(q, 10, mode=O.MODE_REFERENCE)
    assert H.assert_equal_up_to_ties(ic, dc, ir, dr, "grid modes") > 0  # ties do occur here


def test_single_bucket_and_bounds():
    cloud = np.array([[-1.0, -2.0], [-3.0, -0.5], [-2.0, -1.0]], np.float32)
    tree = O.OracleTree(cloud, bucket_size=8)
    t = tree.export()
    assert tree.node_count == 1 and t["cut_dim"][0] == -1 and list(t["buckets"]) == [0, 1, 2]
    # bounds are not computed for a single bucket (nabo/kdtree_cpu.cpp:236-243)
    assert (t["min_bound"] == np.finfo(np.float32).max).all()
    assert (t["max_bound"] == np.finfo(np.float32).tiny).all()
    big = np.concatenate([cloud] * 5)
    t2 = O.OracleTree(big, bucket_size=2).export()
    # all coordinates negative: max bound stays at numeric_limits<float>::min()
    assert (t2["max_bound"] == np.finfo(np.float32).tiny).all()
    assert np.allclose(t2["min_bound"], big.min(axis=0))


def test_argument_errors():
    cloud = np.random.default_rng(0).random((10, 3)).astype(np.float32)
    with pytest.raises(O.OracleError, match="bucket size 1, but must be larger than 2"):
        O.OracleTree(cloud, bucket_size=1)
    with pytest.raises(O.OracleError, match="at least one dimension"):
        O.OracleTree(cloud, dim=0)
    tree = O.OracleTree(cloud)
    with pytest.raises(O.OracleError, match=r"Requesting more points \(10\) than available in cloud minus 1 \(9\)"):
        tree.knn(cloud, 10)
    tree.knn(cloud, 10, option_flags=H.ALLOW_SELF_MATCH)
    with pytest.raises(O.OracleError, match=r"Requesting more points \(11\) than available in cloud \(10\)"):
        tree.knn(cloud, 11, option_flags=H.ALLOW_SELF_MATCH)
    with pytest.raises(O.OracleError, match="Query has less dimensions"):
        tree.knn(cloud[:, :2], 2)
    with pytest.raises(O.OracleError, match="OR-ed value of option flags"):
        tree.knn(cloud, 2, option_flags=4)
