"""Brute force on clouds that stress the float kernel's pre-filter.

The float brute force skips a group of points when |p|^2 - 2 q.p, computed
with fused multiply-adds, is above the query's threshold minus |q|^2 plus a
rounding bound; groups that pass get the reference's distance (separately
rounded squares, nabo/kdtree_cpu.cpp:383-391). These clouds make that bound
matter: points far from the origin at small spacing (|p|^2 much larger than
the distances), coordinates whose squares overflow float, exact ties,
self matches and radius bounds. Results must equal the oracle's brute force
exactly (indices and squared distances, ties to the lower index)."""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _bf(cloud, q, k, flags=0, radius=np.inf, radii=None):
    import libnabo_gb300 as nb
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA)
    gi, gd = s.knn(q, k, 0.0, flags, radius, maxRadii=radii)
    oi, od, _ = O.bf_knn(cloud, q, k, flags, radius, max_radii=radii, mode=O.MODE_CANONICAL)
    return gi, gd, oi, od


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("offset", [1.0e3, 3.0e4])
@pytest.mark.parametrize("k", [1, 5, 16])
def test_far_from_origin(dtype, offset, k):
    rng = np.random.default_rng(int(offset) + k)
    cloud = (offset + rng.random((20000, 3)) * 2.0).astype(dtype)
    q = (cloud[rng.integers(0, cloud.shape[0], 3000)] + rng.normal(0, 1e-3, (3000, 3))).astype(dtype)
    gi, gd, oi, od = _bf(cloud, q, k)
    H.assert_identical(gi, gd, oi, od, f"offset {offset} k={k} {dtype.__name__}")


def test_coordinates_near_float_overflow():
    """|p|^2 overflows for some points (3e19^2 > FLT_MAX): their groups
    go to the exact pass, whose distances overflow the same way as the
    reference's."""
    rng = np.random.default_rng(7)
    small = rng.random((3000, 3))
    big = 1.0e19 + rng.random((3000, 3)) * 1.0e18
    huge = 3.0e19 + rng.random((500, 3)) * 1.0e18
    cloud = np.concatenate([small, big, huge]).astype(np.float32)
    rng.shuffle(cloud)
    q = np.concatenate([small[:400] + 0.01, big[:400] * (1 + 1e-6), huge[:200] * (1 - 1e-6)]).astype(np.float32)
    for k in (1, 6):
        gi, gd, oi, od = _bf(cloud, q, k)
        H.assert_identical(gi, gd, oi, od, f"near overflow k={k}")


def test_ties_self_match_and_radii():
    import libnabo_gb300 as nb
    rng = np.random.default_rng(8)
    cloud = rng.integers(0, 6, (8000, 3)).astype(np.float32)  # many exact duplicates
    q = np.concatenate([cloud[:1500], cloud[1500:3000] + rng.normal(0, 0.2, (1500, 3))]).astype(np.float32)
    for flags in (0, nb.ALLOW_SELF_MATCH):
        gi, gd, oi, od = _bf(cloud, q, 8, flags)
        H.assert_identical(gi, gd, oi, od, f"ties flags={flags}")
    gi, gd, oi, od = _bf(cloud, q, 8, 0, 0.5)
    H.assert_identical(gi, gd, oi, od, "ties, radius 0.5")
    radii = rng.uniform(0.0, 1.5, q.shape[0]).astype(np.float32)
    radii[::7] = np.nan
    gi, gd, oi, od = _bf(cloud, q, 8, 0, np.inf, radii)
    H.assert_identical(gi, gd, oi, od, "ties, per-query radii with NaN entries")
    assert (gi[::7] == -1).all()
