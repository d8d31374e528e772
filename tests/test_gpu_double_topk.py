"""Double searches with 16 or more neighbours per query, whose top-k lists
live in shared memory as binary max-heaps (registers would spill): results
and TOUCH_STATISTICS counts bit-identical to the oracle's canonical
traversal, with a radius, self matches, per-query radii and the learned
form's rerun (nabo/kdtree_cpu.cpp:306-336, 367-447)."""
import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cloud(dim, n, seed):
    from libnabo_gb300 import synthetic as S
    c, centres, sig = S.clusters(n, dim, seed, dtype=np.float64)
    q, _, _ = S.clusters(3000, dim, seed + 1, dtype=np.float64, centres=centres, sigmas=sig)
    return c, q


@pytest.mark.parametrize("dim", [3, 8])
@pytest.mark.parametrize("k", [11, 16, 20, 32])
def test_double_lists_of_16_and_more(dim, k):
    import libnabo_gb300 as nb
    cloud, q = _cloud(dim, 20000, 30 + dim + k)
    tree = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)
    own = cloud[:500]
    for qq, flags, radius in ((q, 0, np.inf), (q, nb.SORT_RESULTS, 0.5), (own, nb.ALLOW_SELF_MATCH, np.inf),
                              (own, 0, np.inf)):
        gi, gd = tree.knn(qq, k, 0.0, flags, radius)
        oi, od, ot = orc.knn(qq, k, 0.0, flags, radius, mode=O.MODE_CANONICAL)
        H.assert_identical(gi, gd, oi, od, f"D={dim} k={k} flags={flags} r={radius}")
        assert tree.touched == ot
    radii = np.random.default_rng(k).uniform(0.0, 2.0, q.shape[0])
    radii[::9] = np.nan
    gi, gd = tree.knn(q, k, 0.0, 0, maxRadii=radii)
    oi, od, ot = orc.knn(q, k, 0.0, 0, max_radii=radii, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"D={dim} k={k} per-query radii")
    assert tree.touched == ot
    gi, gd = tree.knn(q, k, 0.5, 0)
    oi, od, ot = orc.knn(q, k, 0.5, 0, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"D={dim} k={k} eps=0.5")
    assert tree.touched == ot
