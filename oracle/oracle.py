"""CPU oracle for libnabo's kNN path -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper over ``oracle/_build/libnabo_oracle.so`` (built from
``oracle/nabo_oracle.cpp`` by ``oracle/Makefile``). Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference legs
use it, and only as the checker or the timed CPU baseline. The product
(``libnabo_gb300``) never imports it.

Array conventions follow the reference's Eigen layout: a cloud is D x N
column-major, i.e. a C-contiguous numpy array of shape (N, D); result
matrices are k x Q column-major, i.e. numpy arrays of shape (Q, k).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnabo_oracle.so")

MODE_REFERENCE = 0
MODE_CANONICAL = 1
HEAP_LINEAR = 0
HEAP_STL = 1

ALLOW_SELF_MATCH = 1
SORT_RESULTS = 2
TOUCH_STATISTICS = 1

_lib = None


def build() -> str:
    """Compile the oracle shared library (g++ + OpenMP) and return its path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    P = ctypes.c_void_p
    i32, i64, u32 = ctypes.c_int, ctypes.c_int64, ctypes.c_uint
    lib.oracle_last_error.restype = ctypes.c_char_p
    lib.oracle_num_threads.restype = i32
    lib.oracle_set_threads.argtypes = [i32]
    for suf, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
        f = getattr(lib, "oracle_tree_build_" + suf)
        f.restype = P
        f.argtypes = [P, i32, i64, i64, i32, u32]
        getattr(lib, "oracle_tree_free_" + suf).argtypes = [P]
        getattr(lib, "oracle_tree_info_" + suf).argtypes = [P, P]
        getattr(lib, "oracle_tree_export_" + suf).argtypes = [P] * 9
        f = getattr(lib, "oracle_tree_knn_" + suf)
        f.restype = i32
        f.argtypes = [P, P, i32, i64, i64, i32, ct, u32, u32, ct, P, i32, i32, P, P, P]
        f = getattr(lib, "oracle_bf_knn_" + suf)
        f.restype = i32
        f.argtypes = [P, i32, i64, i64, i32, P, i32, i64, i64, i32, u32, u32, ct, P, i32, P, P, P]
    _lib = lib
    return lib


class OracleError(RuntimeError):
    """Argument error reported by the oracle (mirrors Nabo::runtime_error)."""


def _suffix(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    _load().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(_load().oracle_num_threads())


class OracleTree:
    """kd-tree built on the CPU exactly as nabo/kdtree_cpu.cpp:109-272 builds it."""

    def __init__(self, cloud: np.ndarray, dim: int | None = None, bucket_size: int = 8, creation_flags: int = 0):
        lib = _load()
        cloud = np.ascontiguousarray(cloud)
        if cloud.dtype not in (np.float32, np.float64):
            cloud = cloud.astype(np.float32)
        self.dtype = cloud.dtype
        self.suf = _suffix(cloud.dtype)
        n, rows = cloud.shape
        self.cloud = cloud
        self.creation_flags = int(creation_flags)
        dim = rows if dim is None else int(dim)
        h = getattr(lib, "oracle_tree_build_" + self.suf)(_ptr(cloud), rows, n, rows, dim, int(bucket_size))
        if not h:
            raise OracleError(lib.oracle_last_error().decode())
        self._h = ctypes.c_void_p(h)
        info = np.zeros(4, dtype=np.int64)
        getattr(lib, "oracle_tree_info_" + self.suf)(self._h, _ptr(info))
        self.node_count, self.bucket_count, self.dim, self.height = (int(x) for x in info)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            getattr(_lib, "oracle_tree_free_" + self.suf)(h)
            self._h = None

    def export(self):
        """Return the tree as numpy arrays in the reference's pre-order node order."""
        n = self.node_count
        cut_dim = np.zeros(n, np.int32)
        cut_val = np.zeros(n, self.dtype)
        right = np.zeros(n, np.uint32)
        b_start = np.zeros(n, np.uint32)
        b_count = np.zeros(n, np.uint32)
        buckets = np.zeros(self.bucket_count, np.int32)
        min_b = np.zeros(self.dim, self.dtype)
        max_b = np.zeros(self.dim, self.dtype)
        getattr(_load(), "oracle_tree_export_" + self.suf)(
            self._h, _ptr(cut_dim), _ptr(cut_val), _ptr(right), _ptr(b_start), _ptr(b_count), _ptr(buckets),
            _ptr(min_b), _ptr(max_b))
        return dict(cut_dim=cut_dim, cut_val=cut_val, right=right, bucket_start=b_start, bucket_count=b_count,
                    buckets=buckets, min_bound=min_b, max_bound=max_b)

    def knn(self, query: np.ndarray, k: int = 1, epsilon: float = 0.0, option_flags: int = 0,
            max_radius: float = np.inf, max_radii: np.ndarray | None = None, mode: int = MODE_CANONICAL,
            heap: int = HEAP_LINEAR):
        """Search; returns (indices (Q,k) int32, dists2 (Q,k), touched)."""
        lib = _load()
        query = np.ascontiguousarray(query, dtype=self.dtype)
        nq, qrows = query.shape
        idx = np.empty((nq, max(k, 0)), np.int32)
        d2 = np.empty((nq, max(k, 0)), self.dtype)
        touched = np.zeros(1, np.uint64)
        radii = None if max_radii is None else np.ascontiguousarray(max_radii, dtype=self.dtype)
        rc = getattr(lib, "oracle_tree_knn_" + self.suf)(
            self._h, _ptr(query), qrows, nq, qrows, int(k), float(epsilon), int(option_flags), self.creation_flags,
            float(max_radius), _ptr(radii), int(mode), int(heap), _ptr(idx), _ptr(d2), _ptr(touched))
        if rc != 0:
            raise OracleError(lib.oracle_last_error().decode())
        return idx, d2, int(touched[0])


def bf_knn(cloud: np.ndarray, query: np.ndarray, k: int = 1, option_flags: int = 0, max_radius: float = np.inf,
           max_radii: np.ndarray | None = None, dim: int | None = None, mode: int = MODE_CANONICAL,
           creation_flags: int = 0):
    """Brute force (nabo/brute_force_cpu.cpp:63-103); returns (indices, dists2, touched)."""
    lib = _load()
    cloud = np.ascontiguousarray(cloud)
    if cloud.dtype not in (np.float32, np.float64):
        cloud = cloud.astype(np.float32)
    suf = _suffix(cloud.dtype)
    query = np.ascontiguousarray(query, dtype=cloud.dtype)
    n, rows = cloud.shape
    nq, qrows = query.shape
    dim = rows if dim is None else int(dim)
    idx = np.empty((nq, max(k, 0)), np.int32)
    d2 = np.empty((nq, max(k, 0)), cloud.dtype)
    touched = np.zeros(1, np.uint64)
    radii = None if max_radii is None else np.ascontiguousarray(max_radii, dtype=cloud.dtype)
    rc = getattr(lib, "oracle_bf_knn_" + suf)(
        _ptr(cloud), rows, n, rows, dim, _ptr(query), qrows, nq, qrows, int(k), int(option_flags),
        int(creation_flags), float(max_radius), _ptr(radii), int(mode), _ptr(idx), _ptr(d2), _ptr(touched))
    if rc != 0:
        raise OracleError(lib.oracle_last_error().decode())
    return idx, d2, int(touched[0])
