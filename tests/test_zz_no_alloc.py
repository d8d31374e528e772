"""The allocation-free search entry point, through the C ABI.

nabo_cuda_knn_device_noalloc is for callers that must not allocate device
memory once running (a real-time perception loop that fixed its GPU memory
at start-up, or an application that owns all device memory through its own
arena). It keeps its query-ordering scratch in a fixed array inside the
library. Its results must equal those of the regular device entry point,
nabo_cuda_knn_device, and the oracle's, on the same inputs: exactly, as for
every search test here. Two calls in a row check that whatever the array
holds from the previous call does not leak into the next one. The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import helpers as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LIMIT = 262144  # NABO_CUDA_NOALLOC_MAX_QUERIES


def _outputs(nq, k, dtype, device="cuda"):
    import torch
    return (torch.full((nq, k), -7, dtype=torch.int32, device=device),
            torch.full((nq, k), -7.0, dtype=dtype, device=device),
            torch.zeros(1, dtype=torch.int64, device=device))


def _call(lib, fn, handle, tq, k, flags, radius, radii, outs, stream):
    idx, d2, touched = outs
    touched.zero_()
    rc = fn(handle, ctypes.c_void_p(tq.data_ptr()), tq.shape[1], tq.shape[0], tq.shape[1], k, 0.0, flags, radius,
            None if radii is None else ctypes.c_void_p(radii.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
            ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(touched.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, lib.nabo_cuda_last_error().decode()


def _host(outs):
    import torch
    torch.cuda.synchronize()
    idx, d2, touched = outs
    return idx.cpu().numpy(), d2.cpu().numpy(), int(touched.item())


def _cloud(dim, dtype, n, seed):
    rng = np.random.default_rng(seed)
    centers = rng.random((16, dim))
    pts = centers[rng.integers(0, 16, n)] + rng.normal(0, 0.05, (n, dim))
    return pts.astype(dtype)


CASES = [
    # (dtype, dim, k, nq): nq = LIMIT at k = 10 in 3-D and 40000 in 8-D reach
    # the query ordering in the array (the regular search's rule); the rest
    # keep the given order
    (np.float32, 3, 10, LIMIT),
    (np.float32, 3, 1, 1000),
    (np.float64, 3, 10, 5000),
    (np.float32, 2, 5, 3000),
    (np.float32, 8, 10, 40000),
    (np.float64, 8, 16, 2000),
    (np.float32, 16, 4, 1500),
    (np.float32, 3, 64, 3000),
]


@pytest.mark.parametrize("dtype,dim,k,nq", CASES)
def test_no_alloc_search_matches_regular_search_and_oracle(dtype, dim, k, nq):
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import _native

    lib = _native.lib
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    cloud = _cloud(dim, dtype, 30000, seed=dim * 7 + k)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    orc = O.OracleTree(cloud, creation_flags=O.TOUCH_STATISTICS)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(nq + dim)
    q1 = (cloud[rng.integers(0, cloud.shape[0], nq)] + rng.normal(0, 0.02, (nq, dim))).astype(dtype)
    q2 = rng.random((nq, dim)).astype(dtype)
    radii = (rng.random(nq) * 0.1).astype(dtype)
    check_oracle = nq <= 50000
    # two calls in a row on the same fixed array: a scalar radius, then
    # per-query radii over other queries
    for q, flags, radius, rad in ((q1, 0, np.inf, None), (q2, nb.ALLOW_SELF_MATCH, np.inf, radii)):
        tq = torch.from_numpy(q).cuda()
        trad = None if rad is None else torch.from_numpy(rad).cuda()
        reg, na = _outputs(nq, k, tdt), _outputs(nq, k, tdt)
        _call(lib, lib.nabo_cuda_knn_device, s._h, tq, k, flags, radius, trad, reg, stream)
        _call(lib, lib.nabo_cuda_knn_device_noalloc, s._h, tq, k, flags, radius, trad, na, stream)
        ri, rd, rt = _host(reg)
        ni, nd, nt = _host(na)
        H.assert_identical(ni, nd, ri, rd, f"no-alloc vs regular {dtype.__name__} D={dim} k={k} nq={nq}")
        assert nt == rt > 0
        if check_oracle:
            oi, od, ot = orc.knn(q, k, 0.0, flags, radius, max_radii=rad, mode=O.MODE_CANONICAL)
            H.assert_identical(ni, nd, oi, od, f"no-alloc vs oracle {dtype.__name__} D={dim} k={k} nq={nq}")
            assert nt == ot


def test_no_alloc_search_allocates_nothing():
    """Device free memory does not move across no-alloc calls (outputs and
    inputs made beforehand; one call first loads the kernels)."""
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import _native

    lib = _native.lib
    cloud = _cloud(3, np.float32, 50000, seed=3)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(4)
    tq = torch.from_numpy(rng.random((LIMIT, 3)).astype(np.float32)).cuda()
    outs = _outputs(LIMIT, 10, torch.float32)
    _call(lib, lib.nabo_cuda_knn_device_noalloc, s._h, tq, 10, 0, np.inf, None, outs, stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _call(lib, lib.nabo_cuda_knn_device_noalloc, s._h, tq, 10, 0, np.inf, None, outs, stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_no_alloc_search_rejects_batches_above_its_limit():
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import _native

    lib = _native.lib
    cloud = np.random.default_rng(1).random((1000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    tq = torch.zeros((LIMIT + 1, 3), dtype=torch.float32, device="cuda")
    idx = torch.empty((LIMIT + 1, 1), dtype=torch.int32, device="cuda")
    d2 = torch.empty((LIMIT + 1, 1), dtype=torch.float32, device="cuda")
    rc = lib.nabo_cuda_knn_device_noalloc(s._h, ctypes.c_void_p(tq.data_ptr()), 3, LIMIT + 1, 3, 1, 0.0, 0,
                                          float("inf"), None, ctypes.c_void_p(idx.data_ptr()),
                                          ctypes.c_void_p(d2.data_ptr()), None, None)
    assert rc == 1  # NABO_CUDA_ERR_ARGUMENT
    assert "exceed its fixed scratch" in lib.nabo_cuda_last_error().decode()
