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


def _host(shape, dtype, pinned):
    if not pinned:
        return np.zeros(shape, dtype)
    import torch
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
           np.dtype(np.int32): torch.int32}[np.dtype(dtype)]
    return torch.zeros(shape, dtype=tdt).pin_memory().numpy()


def _knn_strided(s, q, k, pad, radii=None, pinned=False):
    """nabo_cuda_knn on columns of q.shape[1] rows stored pad values apart
    (page-locked host buffers with pinned=True)."""
    from libnabo_gb300 import _native
    nq, rows = q.shape
    buf = _host((nq, rows + pad), q.dtype, pinned)
    buf[:, :rows] = q
    idx = _host((nq, k), np.int32, pinned)
    d2 = _host((nq, k), q.dtype, pinned)
    if radii is not None and pinned:
        r = _host(radii.shape, radii.dtype, True)
        r[:] = radii
        radii = r
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


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_pinned_large_call_is_pipelined_and_exact(dtype):
    """Page-locked buffers and 2^18 or more queries: chunks on several
    streams, copies overlapping searches; same results and touched count."""
    nb = _nb()
    rng = np.random.default_rng(11)
    cloud = rng.random((200_000, 3)).astype(dtype)
    nq = 700_001
    q = rng.random((nq, 3)).astype(dtype)
    radii = rng.uniform(0.002, 0.02, nq).astype(dtype)
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    gi, gd, gt = _knn_strided(s, q, 7, pad=2, pinned=True)
    oi, od, ot = orc.knn(q, 7, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, "pipelined")
    assert gt == ot
    gi, gd, gt = _knn_strided(s, q, 7, pad=0, radii=radii, pinned=True)
    oi, od, ot = orc.knn(q, 7, max_radii=radii, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, "pipelined radii")
    assert gt == ot
    hq = _host(q.shape, dtype, True)
    hq[:] = q
    out = (_host((nq, 40), np.int32, True), _host((nq, 40), dtype, True))
    gi, gd = s.knn(hq, 40, out=out)  # k > 32 through the same path
    oi, od, _ = orc.knn(q, 40, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, "pipelined k=40")


@pytest.mark.parametrize("variant", ["bruteforce", "unordered"])
def test_pinned_large_call_unordered_chunks(variant):
    """The pipelined path without a query order: brute force, and the
    kd-tree with query ordering off, searched in plain consecutive chunks."""
    nb = _nb()
    rng = np.random.default_rng(12)
    cloud = rng.random((4000, 3)).astype(np.float32)
    nq = 300_000
    q = rng.random((nq, 3)).astype(np.float32)
    if variant == "bruteforce":
        s = nb.NearestNeighbourSearch(cloud, nb.SearchType.BRUTE_FORCE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    else:
        s = nb.NearestNeighbourSearch(cloud, params={"queryOrdering": 0}, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    gi, gd, gt = _knn_strided(s, q, 6, pad=1, pinned=True)
    oi, od, ot = orc.knn(q, 6, mode=O.MODE_CANONICAL)
    H.assert_identical(gi, gd, oi, od, variant)
    assert gt == (nq * cloud.shape[0] if variant == "bruteforce" else ot)


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


@pytest.mark.parametrize("radii", [False, True], ids=["plain", "radii"])
def test_repeated_pinned_calls_replay_a_graph(radii):
    """A large call repeated with the same page-locked buffers and arguments
    is captured into a CUDA graph on its first repeat and replayed after;
    every call reads the buffers' current contents (new queries and radii
    written in place) and returns the oracle's results and touched count."""
    from libnabo_gb300 import _native
    nb = _nb()
    rng = np.random.default_rng(13)
    cloud = rng.random((150_000, 3)).astype(np.float32)
    nq, k = 300_000, 8
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=H.TOUCH_STATISTICS)
    hq = _host((nq, 3), np.float32, True)
    hr = _host((nq,), np.float32, True) if radii else None
    idx = _host((nq, k), np.int32, True)
    d2 = _host((nq, k), np.float32, True)
    for it in range(4):
        hq[:] = rng.random((nq, 3)).astype(np.float32)
        if radii:
            hr[:] = rng.uniform(0.003, 0.03, nq).astype(np.float32)
        touched = ctypes.c_uint64(0)
        rc = _native.lib.nabo_cuda_knn(s._h, hq.ctypes.data_as(ctypes.c_void_p), 3, nq, 3, k, 0.0, 0,
                                         float("inf"), None if hr is None else hr.ctypes.data_as(ctypes.c_void_p),
                                         idx.ctypes.data_as(ctypes.c_void_p), d2.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.byref(touched))
        assert rc == 0, _native.lib.nabo_cuda_last_error().decode()
        oi, od, ot = orc.knn(hq, k, max_radii=hr, mode=O.MODE_CANONICAL)
        H.assert_identical(idx, d2, oi, od, f"call {it}")
        assert int(touched.value) == ot, it
