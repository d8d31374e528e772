"""libnabo_gb300 -- k-nearest-neighbour search on one NVIDIA GB300.

A drop-in for the kNN path of libnabo 1.1.2. This module mirrors the
reference's Python binding ``pynabo`` (python/nabo.cpp:95-218):
``NearestNeighbourSearch(cloud, searchType, dim, creationOptionFlags,
params)`` and ``.knn(query, k, epsilon, optionFlags, maxRadius)`` returning
``(indices, dists2)``, plus the per-query radii overload of the C++ API
(nabo/nabo.h:351). All compute runs in the CUDA library through the C ABI
of include/nabo_gb300.h; there is no CPU path.

Arrays: a cloud or query set is a C-contiguous numpy array of shape
(n, dim) -- each point's coordinates contiguous, which is the reference's
column-major dim x n layout. Results have shape (nq, k), ascending by
distance; unfound slots hold index -1 and distance +inf.
"""
from __future__ import annotations

import ctypes
import enum

import numpy as np

from ._native import lib as _lib
from ._native import nabo_cuda_params, nabo_cuda_train_params

__all__ = [
    "SearchType", "SearchOptionFlags", "CreationOptionFlags", "NaboError", "NearestNeighbourSearch",
    "InvalidIndex", "ALLOW_SELF_MATCH", "SORT_RESULTS", "TOUCH_STATISTICS", "version", "RadiusModel",
    "RADIUS_MODEL_PARAMS", "RADIUS_MODEL_INPUTS",
]

RADIUS_MODEL_PARAMS = 5313
RADIUS_MODEL_INPUTS = 16

InvalidIndex = -1
# default `dim`: numeric_limits<Index>::max(), clamped to the cloud rows (nabo/nabo.h:360)
_DIM_ALL = 2**31 - 1


class SearchType(enum.IntEnum):
    """nabo/nabo.h:290-299, with the CUDA types after BRUTE_FORCE_CL."""
    BRUTE_FORCE = 0
    KDTREE_LINEAR_HEAP = 1
    KDTREE_TREE_HEAP = 2
    KDTREE_CL_PT_IN_NODES = 3
    KDTREE_CL_PT_IN_LEAVES = 4
    BRUTE_FORCE_CL = 5
    KDTREE_CUDA = 6
    BRUTE_FORCE_CUDA = 7
    SEARCH_TYPE_COUNT = 8


class SearchOptionFlags(enum.IntFlag):
    """nabo/nabo.h:308-312."""
    ALLOW_SELF_MATCH = 1
    SORT_RESULTS = 2


class CreationOptionFlags(enum.IntFlag):
    """nabo/nabo.h:302-305."""
    TOUCH_STATISTICS = 1


ALLOW_SELF_MATCH = int(SearchOptionFlags.ALLOW_SELF_MATCH)
SORT_RESULTS = int(SearchOptionFlags.SORT_RESULTS)
TOUCH_STATISTICS = int(CreationOptionFlags.TOUCH_STATISTICS)

_ERR_NAMES = {1: "argument", 2: "cuda", 3: "unsupported", 4: "internal"}


class NaboError(RuntimeError):
    """Error raised by the library; mirrors Nabo::runtime_error (nabo/nabo.cpp:50-66).

    ``code`` is the C-ABI status (1 argument, 2 CUDA, 3 unsupported, 4 internal).
    """

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code
        self.kind = _ERR_NAMES.get(code, "unknown")


def _check(rc: int) -> None:
    if rc != 0:
        raise NaboError(rc, _lib.nabo_cuda_last_error().decode())


def version() -> str:
    return _lib.nabo_cuda_version().decode()


def measure_fma_peak(dtype=np.float32) -> float:
    """Measured FMA throughput of the current GPU in flop/s (the brute-force
    search's roofline denominator)."""
    out = ctypes.c_double(0.0)
    _check(_lib.nabo_cuda_measure_fma_peak(_dtype_code(np.dtype(dtype)), ctypes.byref(out)))
    return float(out.value)


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.float32:
        return 0
    if dt == np.float64:
        return 1
    raise NaboError(1, f"unsupported scalar type {dt}; use float32 or float64")


def _ptr(a) -> ctypes.c_void_p | None:
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


class NearestNeighbourSearch:
    """A kNN search object on the current CUDA device.

    Mirrors ``pynabo.NearestNeighbourSearch`` (python/nabo.cpp:98-130) and
    ``Nabo::NearestNeighbourSearch<T>::create`` (nabo/nabo.h:360). ``cloud``
    is a numpy array (host) or a CUDA torch tensor (device) of shape
    (n, rows); it is copied into the search object. ``params`` accepts the
    reference's ``bucketSize`` key, ``queryOrdering`` (1 = sort the queries
    of large searches along a Morton curve, the default) and ``traversal``
    (0 or 1 the reference's visit order, 2 the warp packet for exact
    searches without touch statistics).
    """

    def __init__(self, cloud, searchType: int = SearchType.KDTREE_CUDA, dim: int | None = None,
                 creationOptionFlags: int = 0, params: dict | None = None):
        self._h = ctypes.c_void_p()
        p = nabo_cuda_params()
        _lib.nabo_cuda_params_init(ctypes.byref(p))
        for key, val in (params or {}).items():
            if key == "bucketSize":
                p.bucketSize = int(val)
            elif key == "queryOrdering":
                p.queryOrdering = int(val)
            elif key == "traversal":
                p.traversal = int(val)
            elif key == "pipelineChunks":
                p.pipelineChunks = int(val)
            elif key == "splitRule":
                p.splitRule = int(val)
            else:
                raise NaboError(1, f"unknown parameter {key!r}")
        self.searchType = int(searchType)
        self.creationOptionFlags = int(creationOptionFlags)
        if _is_torch(cloud):
            import torch
            if not cloud.is_cuda or cloud.dim() != 2:
                raise NaboError(1, "a torch cloud must be a 2-D CUDA tensor")
            cloud = cloud.contiguous()
            self.dtype = np.dtype(str(cloud.dtype).replace("torch.", ""))
            n, rows = cloud.shape
            dimv = _DIM_ALL if dim is None else int(dim)
            with torch.cuda.device(cloud.device):
                torch.cuda.current_stream().synchronize()
                _check(_lib.nabo_cuda_create_device(
                    _dtype_code(self.dtype), ctypes.c_void_p(cloud.data_ptr()), rows, n, rows, dimv,
                    self.searchType, self.creationOptionFlags, ctypes.byref(p), ctypes.byref(self._h)))
        else:
            cloud = np.asarray(cloud)
            if cloud.ndim != 2:
                raise NaboError(1, "cloud must be a 2-D array (points x coordinates)")
            if cloud.dtype not in (np.float32, np.float64):
                cloud = cloud.astype(np.float64)
            cloud = np.ascontiguousarray(cloud)
            self.dtype = cloud.dtype
            n, rows = cloud.shape
            dimv = _DIM_ALL if dim is None else int(dim)
            _check(_lib.nabo_cuda_create(
                _dtype_code(self.dtype), _ptr(cloud), rows, n, rows, dimv, self.searchType,
                self.creationOptionFlags, ctypes.byref(p), ctypes.byref(self._h)))
        info = (ctypes.c_int64 * 8)()
        _check(_lib.nabo_cuda_get_info(self._h, info))
        self.dim, self.n = int(info[0]), int(info[1])
        self.bucketSize = int(info[5])
        self.nodeCount, self.height = int(info[6]), int(info[7])
        lo = np.zeros(self.dim, self.dtype)
        hi = np.zeros(self.dim, self.dtype)
        _check(_lib.nabo_cuda_get_bounds(self._h, _ptr(lo), _ptr(hi)))
        self.minBound, self.maxBound = lo, hi
        self.touched = 0

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.nabo_cuda_destroy(h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- search -----------------------------------------------------------
    def knn(self, query, k: int = 1, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf,
            maxRadii=None, out=None):
        """k nearest neighbours of each row of ``query``; returns (indices, dists2).

        ``maxRadii`` (one radius per query) selects the reference's per-query
        radius overload (nabo/nabo.h:351); otherwise ``maxRadius`` applies to
        all queries (nabo/nabo.h:338). With TOUCH_STATISTICS the visited-point
        count of the call is left in ``self.touched``. ``out`` may supply the
        (indices, dists2) host arrays (C-contiguous, shape (nq, k)), e.g.
        pinned buffers.
        """
        if _is_torch(query):
            return self.knn_device(query, k, epsilon, optionFlags, maxRadius, maxRadii)
        query = np.ascontiguousarray(np.asarray(query, dtype=self.dtype))
        if query.ndim == 1:
            query = query.reshape(1, -1)
        nq, qrows = query.shape
        kk = int(k)
        if out is None:
            idx = np.empty((nq, max(kk, 0)), np.int32)
            d2 = np.empty((nq, max(kk, 0)), self.dtype)
        else:
            idx, d2 = out
            if (idx.shape != (nq, kk) or d2.shape != (nq, kk) or idx.dtype != np.int32 or d2.dtype != self.dtype
                    or not idx.flags.c_contiguous or not d2.flags.c_contiguous):
                raise NaboError(1, "out arrays must be C-contiguous (nq, k) int32 / scalar arrays")
        radii = None
        if maxRadii is not None:
            radii = np.ascontiguousarray(np.asarray(maxRadii, dtype=self.dtype).reshape(-1))
            if radii.shape[0] != nq:
                # nabo/nabo.cpp:126-127
                raise NaboError(1, f"Maximum radii vector has not the same length ({radii.shape[0]}) "
                                   f"than query has columns ({kk})")
        touched = ctypes.c_uint64(0)
        _check(_lib.nabo_cuda_knn(self._h, _ptr(query), qrows, nq, qrows, kk, float(epsilon), int(optionFlags),
                                  float(maxRadius), _ptr(radii), _ptr(idx), _ptr(d2), ctypes.byref(touched)))
        self.touched = int(touched.value)
        return idx, d2

    def knn_device(self, query, k: int = 1, epsilon: float = 0.0, optionFlags: int = 0,
                   maxRadius: float = np.inf, maxRadii=None, out=None, touched=None, stream=None):
        """Search with CUDA torch tensors, stream-ordered, no host synchronisation.

        ``query`` is an (nq, rows) CUDA tensor; returns (indices, dists2) CUDA
        tensors of shape (nq, k) (or fills ``out``). ``touched`` may be a
        1-element int64 CUDA tensor to which the TOUCH_STATISTICS count is added.
        """
        import torch
        if not query.is_cuda:
            raise NaboError(1, "knn_device needs a CUDA tensor")
        query = query.contiguous()
        nq, qrows = query.shape
        tdt = torch.float32 if self.dtype == np.float32 else torch.float64
        if query.dtype != tdt:
            raise NaboError(1, f"query dtype {query.dtype} does not match the cloud's {tdt}")
        if out is None:
            idx = torch.empty((nq, k), dtype=torch.int32, device=query.device)
            d2 = torch.empty((nq, k), dtype=tdt, device=query.device)
        else:
            idx, d2 = out
        rp = None
        if maxRadii is not None:
            maxRadii = maxRadii.contiguous()
            if maxRadii.numel() != nq:
                raise NaboError(1, f"Maximum radii vector has not the same length ({maxRadii.numel()}) "
                                   f"than query has columns ({k})")
            rp = ctypes.c_void_p(maxRadii.data_ptr())
        st = stream if stream is not None else torch.cuda.current_stream(query.device).cuda_stream
        tp = None if touched is None else ctypes.c_void_p(touched.data_ptr())
        _check(_lib.nabo_cuda_knn_device(self._h, ctypes.c_void_p(query.data_ptr()), qrows, nq, qrows, int(k),
                                         float(epsilon), int(optionFlags), float(maxRadius), rp,
                                         ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(d2.data_ptr()), tp,
                                         ctypes.c_void_p(st)))
        return idx, d2

    def profile(self, enable: bool = True) -> None:
        """Bracket the search kernel of later device searches with CUDA events."""
        _check(_lib.nabo_cuda_profile(self._h, 1 if enable else 0))

    def last_kernel_ms(self) -> float:
        """Duration of the last device search's kernel (waits for it)."""
        ms = ctypes.c_float(0.0)
        _check(_lib.nabo_cuda_last_kernel_ms(self._h, ctypes.byref(ms)))
        return float(ms.value)

    def export_tree(self) -> dict:
        """The kd-tree as numpy arrays in pre-order (for parity checks)."""
        n = self.nodeCount
        cut_dim = np.zeros(n, np.int32)
        cut_val = np.zeros(n, self.dtype)
        right = np.zeros(n, np.uint32)
        b_start = np.zeros(n, np.uint32)
        b_count = np.zeros(n, np.uint32)
        buckets = np.zeros(self.n, np.int32)
        _check(_lib.nabo_cuda_export_tree(self._h, _ptr(cut_dim), _ptr(cut_val), _ptr(right), _ptr(b_start),
                                          _ptr(b_count), _ptr(buckets)))
        return dict(cut_dim=cut_dim, cut_val=cut_val, right=right, bucket_start=b_start, bucket_count=b_count,
                    buckets=buckets)

    # Factory helpers named after the reference's (nabo/nabo.h:360-386).
    @classmethod
    def create(cls, cloud, dim=None, preferedType=SearchType.KDTREE_CUDA, creationOptionFlags=0,
               additionalParameters=None):
        return cls(cloud, preferedType, dim, creationOptionFlags, additionalParameters)

    @classmethod
    def createKDTreeCUDA(cls, cloud, dim=None, creationOptionFlags=0, additionalParameters=None):
        return cls(cloud, SearchType.KDTREE_CUDA, dim, creationOptionFlags, additionalParameters)

    @classmethod
    def createBruteForceCUDA(cls, cloud, dim=None, creationOptionFlags=0):
        return cls(cloud, SearchType.BRUTE_FORCE_CUDA, dim, creationOptionFlags, None)


def _torch_device_array(x, dtype):
    """A CUDA tensor of `x` (numpy or torch) with the given torch dtype."""
    import torch
    if _is_torch(x):
        return x.to(device="cuda" if not x.is_cuda else x.device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype)


class RadiusModel:
    """Learned per-query search radius for a KDTREE_CUDA search object.

    A small BF16 network, trained on the GPU by the library's own kernels,
    predicts log(d_k) for a query (from its coordinates and, in 3-D, the
    occupancy of the coarse voxels around it). ``knn`` searches with the
    per-query radius ``safety * exp(prediction)`` and searches again,
    without the bound, every query that found fewer than k neighbours inside
    it, so the results equal ``NearestNeighbourSearch.knn``. ``fallbacks``
    holds how many queries the last search had to repeat.
    """

    def __init__(self, search: NearestNeighbourSearch, train_queries, k: int, optionFlags: int = 0,
                 maxRadius: float = np.inf, epochs: int = 30, batch: int = 4096, lr: float = 3e-3,
                 safety: float = 1.2, seed: int = 1234, targetMissRate: float = 0.01):
        import torch
        self.search = search
        self.k = int(k)
        self._m = ctypes.c_void_p()
        tdt = torch.float32 if search.dtype == np.float32 else torch.float64
        tq = _torch_device_array(train_queries, tdt)
        n, rows = tq.shape
        p = nabo_cuda_train_params()
        _lib.nabo_cuda_train_params_init(ctypes.byref(p))
        p.epochs, p.batch, p.lr, p.safety, p.seed = int(epochs), int(batch), float(lr), float(safety), int(seed)
        p.targetMissRate = float(targetMissRate)
        torch.cuda.synchronize()
        _check(_lib.nabo_cuda_radius_model_train(search._h, ctypes.c_void_p(tq.data_ptr()), rows, n, rows, self.k,
                                                 int(optionFlags), float(maxRadius), ctypes.byref(p),
                                                 ctypes.byref(self._m)))
        self.fallbacks = 0
        self.touched = 0

    def close(self) -> None:
        m = getattr(self, "_m", None)
        if m is not None and m.value:
            _lib.nabo_cuda_radius_model_destroy(m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def meta(self) -> dict:
        meta = (ctypes.c_float * 16)()
        _check(_lib.nabo_cuda_radius_model_get(self._m, None, meta))
        return dict(mu=meta[0], sigma=meta[1], safety=meta[2], k=int(meta[3]), train_loss=meta[4],
                    train_samples=int(meta[5]), inputs=int(meta[6]), margin=meta[7], voxel=meta[8])

    def get_params(self):
        params = np.zeros(RADIUS_MODEL_PARAMS, np.float32)
        meta = np.zeros(16, np.float32)
        _check(_lib.nabo_cuda_radius_model_get(self._m, _ptr(params), _ptr(meta)))
        return params, meta

    def set_params(self, params, meta=None):
        params = np.ascontiguousarray(params, dtype=np.float32)
        if params.shape != (RADIUS_MODEL_PARAMS,):
            raise NaboError(1, f"expected {RADIUS_MODEL_PARAMS} parameters")
        m = None if meta is None else np.ascontiguousarray(meta, dtype=np.float32)
        _check(_lib.nabo_cuda_radius_model_set(self._m, _ptr(params), _ptr(m)))

    def save(self, path: str) -> None:
        params, meta = self.get_params()
        np.savez(path, params=params, meta=meta)

    def load(self, path: str) -> None:
        with np.load(path) as z:
            self.set_params(z["params"], z["meta"])

    def _tq(self, query):
        import torch
        tdt = torch.float32 if self.search.dtype == np.float32 else torch.float64
        return _torch_device_array(query, tdt)

    def features(self, query):
        """Network inputs (nq, 16) float32 CUDA tensor."""
        import torch
        tq = self._tq(query)
        nq, rows = tq.shape
        X = torch.empty((nq, RADIUS_MODEL_INPUTS), dtype=torch.float32, device=tq.device)
        st = torch.cuda.current_stream(tq.device).cuda_stream
        _check(_lib.nabo_cuda_radius_model_features_device(self._m, ctypes.c_void_p(tq.data_ptr()), rows, nq, rows,
                                                           ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(st)))
        return X

    def predict(self, query, maxRadius: float = np.inf, raw: bool = False):
        """Per-query radii (CUDA tensor); with raw=True also the standardised outputs."""
        import torch
        tq = self._tq(query)
        nq, rows = tq.shape
        radii = torch.empty(nq, dtype=tq.dtype, device=tq.device)
        out = torch.empty(nq, dtype=torch.float32, device=tq.device) if raw else None
        st = torch.cuda.current_stream(tq.device).cuda_stream
        _check(_lib.nabo_cuda_radius_model_predict_device(
            self._m, ctypes.c_void_p(tq.data_ptr()), rows, nq, rows, float(maxRadius),
            ctypes.c_void_p(radii.data_ptr()), None if out is None else ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(st)))
        return (radii, out) if raw else radii

    def gradients(self, features, targets):
        """(grad[RADIUS_MODEL_PARAMS], summed squared error) of the MSE over the samples."""
        import torch
        X = _torch_device_array(features, torch.float32)
        Y = _torch_device_array(targets, torch.float32)
        grad = np.zeros(RADIUS_MODEL_PARAMS, np.float32)
        loss = ctypes.c_float(0.0)
        torch.cuda.synchronize()
        _check(_lib.nabo_cuda_radius_model_gradients(self._m, ctypes.c_void_p(X.data_ptr()),
                                                     ctypes.c_void_p(Y.data_ptr()), X.shape[0], _ptr(grad),
                                                     ctypes.byref(loss)))
        return grad, float(loss.value)

    def knn(self, query, k: int | None = None, epsilon: float = 0.0, optionFlags: int = 0,
            maxRadius: float = np.inf, out=None):
        """Learned search with host arrays; returns (indices, dists2)."""
        k = self.k if k is None else int(k)
        if _is_torch(query):
            return self.knn_device(query, k, epsilon, optionFlags, maxRadius)
        query = np.ascontiguousarray(np.asarray(query, dtype=self.search.dtype))
        nq, qrows = query.shape
        if out is None:
            idx = np.empty((nq, k), np.int32)
            d2 = np.empty((nq, k), self.search.dtype)
        else:
            idx, d2 = out
        touched = ctypes.c_uint64(0)
        fb = ctypes.c_int64(0)
        _check(_lib.nabo_cuda_knn_learned(self.search._h, self._m, _ptr(query), qrows, nq, qrows, k, float(epsilon),
                                          int(optionFlags), float(maxRadius), _ptr(idx), _ptr(d2),
                                          ctypes.byref(touched), ctypes.byref(fb)))
        self.touched = int(touched.value)
        self.fallbacks = int(fb.value)
        return idx, d2

    def knn_device(self, query, k: int | None = None, epsilon: float = 0.0, optionFlags: int = 0,
                   maxRadius: float = np.inf, out=None, touched=None, fallbacks=None, stream=None):
        """Learned search with CUDA tensors, stream-ordered; returns (indices, dists2)."""
        import torch
        k = self.k if k is None else int(k)
        query = query.contiguous()
        nq, qrows = query.shape
        if out is None:
            idx = torch.empty((nq, k), dtype=torch.int32, device=query.device)
            d2 = torch.empty((nq, k), dtype=query.dtype, device=query.device)
        else:
            idx, d2 = out
        st = stream if stream is not None else torch.cuda.current_stream(query.device).cuda_stream
        _check(_lib.nabo_cuda_knn_learned_device(
            self.search._h, self._m, ctypes.c_void_p(query.data_ptr()), qrows, nq, qrows, k, float(epsilon),
            int(optionFlags), float(maxRadius), ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(d2.data_ptr()),
            None if touched is None else ctypes.c_void_p(touched.data_ptr()),
            None if fallbacks is None else ctypes.c_void_p(fallbacks.data_ptr()), ctypes.c_void_p(st)))
        return idx, d2


class BatchRadiusModel:
    """A learned-radius model for batched searches (one per dimension and
    scalar type), made by :meth:`BatchSearch.train_radius_model`."""

    def __init__(self, handle):
        self._m = handle

    def close(self) -> None:
        m = getattr(self, "_m", None)
        if m is not None and m.value:
            _lib.nabo_cuda_radius_model_destroy(m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def meta(self) -> dict:
        meta = (ctypes.c_float * 16)()
        _check(_lib.nabo_cuda_radius_model_get(self._m, None, meta))
        return dict(mu=meta[0], sigma=meta[1], safety=meta[2], k=int(meta[3]), train_loss=meta[4],
                    train_samples=int(meta[5]), inputs=int(meta[6]), margin=meta[7])

    def gradients(self, features, targets):
        """(grad, summed squared error) of the MSE over given inputs and targets."""
        import torch
        X = _torch_device_array(features, torch.float32)
        Y = _torch_device_array(targets, torch.float32)
        grad = np.zeros(RADIUS_MODEL_PARAMS, np.float32)
        loss = ctypes.c_float(0.0)
        torch.cuda.synchronize()
        _check(_lib.nabo_cuda_radius_model_gradients(self._m, ctypes.c_void_p(X.data_ptr()),
                                                     ctypes.c_void_p(Y.data_ptr()), X.shape[0], _ptr(grad),
                                                     ctypes.byref(loss)))
        return grad, float(loss.value)

    def get_params(self):
        params = np.zeros(RADIUS_MODEL_PARAMS, np.float32)
        meta = np.zeros(16, np.float32)
        _check(_lib.nabo_cuda_radius_model_get(self._m, _ptr(params), _ptr(meta)))
        return params, meta


class BatchSearch:
    """Many clouds of uneven sizes built and searched together.

    The clouds are stored back to back in one (total_points, dim) CUDA tensor
    (cloud c = the next ``point_counts[c]`` rows); each gets the kd-tree the
    reference builds for it alone, all built in one forest build, and all
    queries (back to back likewise, ``query_counts[c]`` rows for cloud c) are
    searched by one kernel launch, each with its cloud's ``k``. ``run``
    captures build + search into a CUDA graph on first use and replays it.
    Results come back flat: cloud c's (nq_c, k_c) block after the earlier
    ones; ``split`` cuts them per cloud. Self matches are not allowed.
    """

    def __init__(self, point_counts, dim: int = 3, dtype=np.float32, bucketSize: int = 8, threadsPerBlock: int = 128,
                 maxLevels: int = 48, pipelineChunks: int = 0, splitRule: int = 0, lanesPerQuery: int = 1):
        counts = np.ascontiguousarray(np.asarray(point_counts, dtype=np.int64))
        self.point_counts = counts
        self.dim = int(dim)
        self.dtype = np.dtype(dtype)
        self._b = ctypes.c_void_p()
        p = nabo_cuda_params()
        _lib.nabo_cuda_params_init(ctypes.byref(p))
        p.bucketSize = int(bucketSize)
        p.threadsPerBlock = int(threadsPerBlock)
        p.pipelineChunks = int(pipelineChunks)
        p.splitRule = int(splitRule)
        p.lanesPerQuery = int(lanesPerQuery)
        _check(_lib.nabo_cuda_batch_create(_dtype_code(self.dtype), self.dim, len(counts), _ptr(counts),
                                           ctypes.byref(p), int(maxLevels), ctypes.byref(self._b)))
        self.query_counts = None
        self.k = None

    def close(self) -> None:
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            _lib.nabo_cuda_batch_destroy(b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_queries(self, query_counts, k) -> None:
        qc = np.ascontiguousarray(np.asarray(query_counts, dtype=np.int64))
        kk = np.ascontiguousarray(np.broadcast_to(np.asarray(k, dtype=np.int32), qc.shape))
        _check(_lib.nabo_cuda_batch_set_queries(self._b, _ptr(qc), _ptr(kk)))
        self.query_counts, self.k = qc, kk
        self.result_entries = int(np.sum(qc * kk))

    def _outputs(self, device):
        import torch
        tdt = torch.float32 if self.dtype == np.float32 else torch.float64
        return (torch.empty(self.result_entries, dtype=torch.int32, device=device),
                torch.empty(self.result_entries, dtype=tdt, device=device))

    def build(self, clouds, stream=None) -> None:
        import torch
        st = stream if stream is not None else torch.cuda.current_stream(clouds.device).cuda_stream
        _check(_lib.nabo_cuda_batch_build_device(self._b, ctypes.c_void_p(clouds.data_ptr()), ctypes.c_void_p(st)))

    def knn(self, queries, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf, out=None,
            stream=None):
        import torch
        idx, d2 = out if out is not None else self._outputs(queries.device)
        st = stream if stream is not None else torch.cuda.current_stream(queries.device).cuda_stream
        _check(_lib.nabo_cuda_batch_knn_device(self._b, ctypes.c_void_p(queries.data_ptr()), float(epsilon),
                                               int(optionFlags), float(maxRadius), ctypes.c_void_p(idx.data_ptr()),
                                               ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(st)))
        return idx, d2

    def knn_radii(self, queries, radii, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf,
                  out=None, fallbacks=None, stream=None):
        """Search with a radius per query (CUDA tensor, one per query row);
        a query whose radius is below ``maxRadius`` and that finds fewer than
        its cloud's k neighbours is searched again with ``maxRadius`` alone,
        counted in ``fallbacks`` (an int32 CUDA tensor of one element, added
        to) when given."""
        import torch
        idx, d2 = out if out is not None else self._outputs(queries.device)
        st = stream if stream is not None else torch.cuda.current_stream(queries.device).cuda_stream
        fb = ctypes.c_void_p(fallbacks.data_ptr()) if fallbacks is not None else None
        _check(_lib.nabo_cuda_batch_knn_radii_device(self._b, ctypes.c_void_p(queries.data_ptr()),
                                                     ctypes.c_void_p(radii.data_ptr()), float(epsilon),
                                                     int(optionFlags), float(maxRadius),
                                                     ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(d2.data_ptr()),
                                                     fb, ctypes.c_void_p(st)))
        return idx, d2

    def train_radius_model(self, queries, dists2, epochs: int = 30, batch: int = 4096, lr: float = 3e-3,
                           safety: float = 1.2, seed: int = 1234, targetMissRate: float = 0.01):
        """A learned-radius model for batches of this dimension and scalar
        type, from training queries laid out by the current query plan
        (CUDA tensor) and their exact squared distances (the ``dists2`` of
        ``knn`` on them). Returns a :class:`BatchRadiusModel`."""
        import torch
        p = nabo_cuda_train_params()
        _lib.nabo_cuda_train_params_init(ctypes.byref(p))
        p.epochs, p.batch, p.lr, p.safety, p.seed = int(epochs), int(batch), float(lr), float(safety), int(seed)
        p.targetMissRate = float(targetMissRate)
        m = ctypes.c_void_p()
        torch.cuda.synchronize()
        _check(_lib.nabo_cuda_batch_radius_model_train(self._b, ctypes.c_void_p(queries.data_ptr()),
                                                       ctypes.c_void_p(dists2.data_ptr()), ctypes.byref(p),
                                                       ctypes.byref(m)))
        return BatchRadiusModel(m)

    def predict_radii(self, model, queries, maxRadius: float = np.inf, raw: bool = False):
        """A batched model's radius per query (CUDA tensor); with raw=True also
        its standardised outputs."""
        import torch
        radii = torch.empty(queries.shape[0], dtype=queries.dtype, device=queries.device)
        out = torch.empty(queries.shape[0], dtype=torch.float32, device=queries.device) if raw else None
        st = torch.cuda.current_stream(queries.device).cuda_stream
        _check(_lib.nabo_cuda_batch_radius_model_predict_device(
            self._b, model._m, ctypes.c_void_p(queries.data_ptr()), float(maxRadius),
            ctypes.c_void_p(radii.data_ptr()), None if out is None else ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(st)))
        return (radii, out) if raw else radii

    def radius_features(self, model, queries):
        """A batched model's network inputs (nq, 16) float32 CUDA tensor."""
        import torch
        X = torch.empty((queries.shape[0], RADIUS_MODEL_INPUTS), dtype=torch.float32, device=queries.device)
        st = torch.cuda.current_stream(queries.device).cuda_stream
        _check(_lib.nabo_cuda_batch_radius_model_features_device(self._b, model._m,
                                                                 ctypes.c_void_p(queries.data_ptr()),
                                                                 ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(st)))
        return X

    def knn_learned(self, model, queries, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf,
                    out=None, fallbacks=None, stream=None):
        """Search with the model's radius per query; results equal ``knn``'s.
        ``fallbacks`` (int32 CUDA tensor of one element) receives how many
        queries were searched again."""
        import torch
        idx, d2 = out if out is not None else self._outputs(queries.device)
        st = stream if stream is not None else torch.cuda.current_stream(queries.device).cuda_stream
        fb = ctypes.c_void_p(fallbacks.data_ptr()) if fallbacks is not None else None
        _check(_lib.nabo_cuda_batch_knn_learned_device(self._b, model._m, ctypes.c_void_p(queries.data_ptr()),
                                                       float(epsilon), int(optionFlags), float(maxRadius),
                                                       ctypes.c_void_p(idx.data_ptr()),
                                                       ctypes.c_void_p(d2.data_ptr()), fb, ctypes.c_void_p(st)))
        return idx, d2

    def run(self, clouds, queries, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf,
            out=None, stream=None):
        """Build + search as one CUDA graph launch (captured on first use)."""
        import torch
        idx, d2 = out if out is not None else self._outputs(queries.device)
        st = stream if stream is not None else torch.cuda.current_stream(queries.device).cuda_stream
        _check(_lib.nabo_cuda_batch_run(self._b, ctypes.c_void_p(clouds.data_ptr()),
                                        ctypes.c_void_p(queries.data_ptr()), float(epsilon), int(optionFlags),
                                        float(maxRadius), ctypes.c_void_p(idx.data_ptr()),
                                        ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(st)))
        return idx, d2

    def run_host(self, clouds, queries, epsilon: float = 0.0, optionFlags: int = 0, maxRadius: float = np.inf,
                 out=None):
        """Build + search from host arrays ((total_points, dim) and
        (total_queries, dim), C order) into host result arrays; returns when
        they are filled. With page-locked arrays (e.g. pinned torch tensors'
        ``.numpy()``) the copies overlap the build and search inside one CUDA
        graph (``pipelineChunks`` cloud groups, 0 = 8)."""
        if self.query_counts is None:
            raise NaboError(1, "call set_queries first")
        c = np.ascontiguousarray(clouds, dtype=self.dtype)
        q = np.ascontiguousarray(queries, dtype=self.dtype)
        if c.shape != (int(self.point_counts.sum()), self.dim):
            raise NaboError(1, f"clouds must be ({int(self.point_counts.sum())}, {self.dim})")
        if q.shape != (int(self.query_counts.sum()), self.dim):
            raise NaboError(1, f"queries must be ({int(self.query_counts.sum())}, {self.dim})")
        if out is None:
            out = (np.empty(self.result_entries, np.int32), np.empty(self.result_entries, self.dtype))
        idx, d2 = out
        if (idx.dtype != np.int32 or d2.dtype != self.dtype or idx.size != self.result_entries
                or d2.size != self.result_entries or not idx.flags.c_contiguous or not d2.flags.c_contiguous):
            raise NaboError(1, f"out must be contiguous int32 and {self.dtype} arrays of {self.result_entries} entries")
        _check(_lib.nabo_cuda_batch_run_host(self._b, _ptr(c), _ptr(q), float(epsilon), int(optionFlags),
                                             float(maxRadius), _ptr(idx), _ptr(d2)))
        return idx, d2

    def status(self) -> dict:
        info = (ctypes.c_int64 * 8)()
        _check(_lib.nabo_cuda_batch_status(self._b, info))
        # bit 4 (a tree taller than the search kernels' stacks, searched with
        # stacks in global memory) is informational
        return dict(ok=(info[0] & ~4) == 0, flags=int(info[0]), nodes=int(info[1]), height=int(info[2]),
                    levels=int(info[3]), results=int(info[4]), queries=int(info[5]), points=int(info[6]),
                    clouds=int(info[7]))

    def split(self, flat):
        """Per-cloud (nq_c, k_c) views of a flat result array."""
        outs, o = [], 0
        for nq, k in zip(self.query_counts, self.k):
            outs.append(flat[o:o + nq * k].reshape(nq, k))
            o += nq * k
        return outs

    def export_tree(self, cloud: int) -> dict:
        count = ctypes.c_int64(0)
        _check(_lib.nabo_cuda_batch_export_tree(self._b, int(cloud), ctypes.byref(count), None, None, None, None,
                                                None, None))
        n = int(count.value)
        cut_dim = np.zeros(n, np.int32)
        cut_val = np.zeros(n, self.dtype)
        right = np.zeros(n, np.uint32)
        b_start = np.zeros(n, np.uint32)
        b_count = np.zeros(n, np.uint32)
        buckets = np.zeros(int(self.point_counts[cloud]), np.int32)
        _check(_lib.nabo_cuda_batch_export_tree(self._b, int(cloud), ctypes.byref(count), _ptr(cut_dim),
                                                _ptr(cut_val), _ptr(right), _ptr(b_start), _ptr(b_count),
                                                _ptr(buckets)))
        return dict(cut_dim=cut_dim, cut_val=cut_val, right=right, bucket_start=b_start, bucket_count=b_count,
                    buckets=buckets)
