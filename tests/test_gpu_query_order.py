"""Searches large enough to sort their queries first (the stable radix sort
over 2048-key tiles: by Morton code up to 3 dimensions, by home leaf above),
at query counts on and just off the tile edges: every query answered, and
answers and TOUCH_STATISTICS counts identical to the oracle's canonical
traversal (nabo/kdtree_cpu.cpp:306-336, 367-447). The order only changes
timing; a sort that lost or repeated a key would leave queries unanswered or
answered twice."""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TILE = 2048


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("nq", [128 * TILE, 128 * TILE + 1, 130 * TILE - 1], ids=["edge", "edge+1", "edge-1"])
def test_morton_ordered_searches(dim, nq):
    import libnabo_gb300 as nb
    rng = np.random.default_rng(1000 * dim + nq % 7)
    cloud = rng.random((20_000, dim)).astype(np.float32)
    q = rng.random((nq, dim)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)
    gi, gd = s.knn(q, 10, 0.0, 0)
    oi, od, ot = orc.knn(q, 10, 0.0, 0, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"D={dim} nq={nq}")
    assert s.touched == ot


@pytest.mark.parametrize("nq", [16 * TILE, 16 * TILE + 1, 20 * TILE + 5])
def test_leaf_ordered_searches(nq):
    import libnabo_gb300 as nb
    from libnabo_gb300 import synthetic as S
    cloud, centres, sig = S.clusters(30_000, 8, 77, dtype=np.float32)
    q, _, _ = S.clusters(nq, 8, 78, dtype=np.float32, centres=centres, sigmas=sig)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)
    gi, gd = s.knn(q, 10, 0.0, 0)
    oi, od, ot = orc.knn(q, 10, 0.0, 0, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"D=8 nq={nq}")
    assert s.touched == ot
