"""The allocation-free search entry point, through the C ABI.

nabo_cuda_knn_device_noalloc is for callers that must not allocate device
memory once running (a real-time perception loop that fixed its GPU memory
at start-up, or an application that owns all device memory through its own
arena). It keeps its query-ordering scratch in a fixed array inside the
library. Its results must equal those of the regular device entry point,
nabo_cuda_knn_device, on the same inputs: exactly, as for every search test
here. Two calls in a row check that whatever the array holds from the
previous call does not leak into the next one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _search(lib, fn, handle, tq, k, flags, radius, stream):
    import torch
    nq = tq.shape[0]
    idx = torch.full((nq, k), -7, dtype=torch.int32, device=tq.device)
    d2 = torch.full((nq, k), -7.0, dtype=tq.dtype, device=tq.device)
    touched = torch.zeros(1, dtype=torch.int64, device=tq.device)
    rc = fn(handle, ctypes.c_void_p(tq.data_ptr()), tq.shape[1], nq, tq.shape[1], k, 0.0, flags, radius, None,
            ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(touched.data_ptr()),
            ctypes.c_void_p(stream))
    assert rc == 0, lib.nabo_cuda_last_error().decode()
    torch.cuda.synchronize()
    return idx.cpu().numpy(), d2.cpu().numpy(), int(touched.item())


def test_no_alloc_search_matches_regular_search():
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import _native

    lib = _native.lib
    rng = np.random.default_rng(2024)
    cloud = rng.random((60000, 3), dtype=np.float64).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud, nb.SearchType.KDTREE_CUDA, creationOptionFlags=nb.TOUCH_STATISTICS)
    stream = torch.cuda.current_stream().cuda_stream
    cases = [
        (rng.random((40000, 3), dtype=np.float64).astype(np.float32), 10, 0, np.inf),
        (rng.random((25000, 3), dtype=np.float64).astype(np.float32), 5, nb.ALLOW_SELF_MATCH, 0.02),
    ]
    for q, k, flags, radius in cases:  # two calls in a row on the same fixed scratch
        tq = torch.from_numpy(q).cuda()
        ri, rd, rt = _search(lib, lib.nabo_cuda_knn_device, s._h, tq, k, flags, radius, stream)
        ni, nd, nt = _search(lib, lib.nabo_cuda_knn_device_noalloc, s._h, tq, k, flags, radius, stream)
        assert np.array_equal(ni, ri)
        assert np.array_equal(nd, rd)
        assert nt == rt > 0


def test_no_alloc_search_rejects_batches_above_its_limit():
    import torch

    import libnabo_gb300 as nb
    from libnabo_gb300 import _native

    lib = _native.lib
    limit = 262144  # NABO_CUDA_NOALLOC_MAX_QUERIES
    cloud = np.random.default_rng(1).random((1000, 3)).astype(np.float32)
    s = nb.NearestNeighbourSearch(cloud)
    tq = torch.zeros((limit + 1, 3), dtype=torch.float32, device="cuda")
    idx = torch.empty((limit + 1, 1), dtype=torch.int32, device="cuda")
    d2 = torch.empty((limit + 1, 1), dtype=torch.float32, device="cuda")
    rc = lib.nabo_cuda_knn_device_noalloc(s._h, ctypes.c_void_p(tq.data_ptr()), 3, limit + 1, 3, 1, 0.0, 0,
                                          float("inf"), None, ctypes.c_void_p(idx.data_ptr()),
                                          ctypes.c_void_p(d2.data_ptr()), None, None)
    assert rc == 1  # NABO_CUDA_ERR_ARGUMENT
    assert "exceed its fixed scratch" in lib.nabo_cuda_last_error().decode()
