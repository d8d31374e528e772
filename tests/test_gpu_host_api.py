"""The host-buffer search (nabo_cuda_knn): small calls go through the
object's pinned staging blocks, large ones through pool allocations, and a
call made while another thread holds the staging takes the general path.
All three give the oracle's results, with strided query columns, per-query
radii and the TOUCH_STATISTICS count."""
import ctypes
import threading

import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


def _knn_strided(s, q, k, pad, radii=None):
    """nabo_cuda_knn on columns of q.shape[1] rows stored pad values apart."""
    from libnabo_gb300 import _native
    nq, rows = q.shape
    buf = np.zeros((nq, rows + pad), q.dtype)
    buf[:, :rows] = q
    idx = np.empty((nq, k), np.int32)
    d2 = np.empty((nq, k), q.dtype)
    touched = ctypes.c_uint64(0)
    rptr = None if radii is None else radii.ctypes.data_as(ctypes.c_void_p)
    rc = _native.lib.nabo_cuda_knn(s._h, buf.ctypes.data_as(ctypes.c_void_p), rows, nq, rows + pad, k, 0.0, 0,
                                     float("inf"), rptr, idx.ctypes.data_as(ctypes.c_void_p),
                                     d2.ctypes.data_as(ctypes.c_void_p), ctypes.byref(touched))
    assert rc == 0, _native.lib.nabo_cuda_last_error().decode()
    return idx, d2, int(touched.value)


@pytest.mark.parametrize("nq", [1, 700, 300_000], ids=["one", "staged", "general"])
def test_strided_queries_match_oracle(nq):
    nb = _nb()
    rng = np.random.default_rng(nq)
    cloud = rng.random((50_000, 3)).astype(np.float32)
    q = rng.random((nq, 3)).astype(np.float32)
    radii = rng.uniform(0.005, 0.05, nq).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    gi, gd, gt = _knn_strided(s, q, 10, pad=3)
    oi, od, ot = orc.knn(q, 10, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"strided nq={nq}")
    assert gt == ot
    gi, gd, gt = _knn_strided(s, q, 10, pad=1, radii=radii)
    oi, od, ot = orc.knn(q, 10, max_radii=radii, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, f"strided radii nq={nq}")
    assert gt == ot


def test_concurrent_calls_on_one_object():
    nb = _nb()
    rng = np.random.default_rng(3)
    cloud = rng.random((40_000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    qs = [rng.random((int(n), 3)).astype(np.float32) for n in rng.integers(1, 3000, 24)]
    expect = [O.OracleTree(cloud).knn(q, 8, mode=O.MODE_CANONICAL)[:2] for q in qs]
    got = [None] * len(qs)
    errors = []

    def work(lo):
        try:
            for _ in range(5):
                for i in range(lo, len(qs), 4):
                    got[i] = s.knn(qs[i], 8)
        except Exception as e:  # noqa: BLE001 -- reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i, (oi, od) in enumerate(expect):
        H.assert_identical(got[i][0], got[i][1], oi, od, f"thread call {i}")


def test_single_point_calls():
    """One query per call (the reference's single-vector knn, nabo/nabo.h:325)."""
    nb = _nb()
    rng = np.random.default_rng(4)
    cloud = rng.random((20_000, 3))
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    for i in range(50):
        q = rng.random(3)
        gi, gd = s.knn(q, 5, 0.0, 0, 0.1)
        oi, od, ot = orc.knn(q.reshape(1, 3), 5, 0.0, 0, 0.1, mode=O.MODE_CANONICAL)
        H.assert_identical(gi, gd, oi, od, f"single point {i}")
        assert s.touched == ot
