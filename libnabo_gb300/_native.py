"""ctypes binding of the C ABI declared in include/nabo_gb300.h.

Loads the in-tree ``libnabo_gb300/lib/libnabo_gb300.so`` on first use.
There is no fallback: if the library is missing or fails to load, the first
call raises, naming the build command.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libnabo_gb300.so")

# Every symbol include/nabo_gb300.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U = ctypes.c_uint
_D = ctypes.c_double
SIGNATURES = {
    "nabo_cuda_params_init": (None, [_P]),
    "nabo_cuda_create": (_I, [_I, _P, _I, _I64, _I64, _I, _I, _U, _P, _P]),
    "nabo_cuda_create_device": (_I, [_I, _P, _I, _I64, _I64, _I, _I, _U, _P, _P]),
    "nabo_cuda_destroy": (_I, [_P]),
    "nabo_cuda_knn": (_I, [_P, _P, _I, _I64, _I64, _I, _D, _U, _D, _P, _P, _P, _P]),
    "nabo_cuda_knn_device": (_I, [_P, _P, _I, _I64, _I64, _I, _D, _U, _D, _P, _P, _P, _P, _P]),
    "nabo_cuda_knn_device_noalloc": (_I, [_P, _P, _I, _I64, _I64, _I, _D, _U, _D, _P, _P, _P, _P, _P]),
    "nabo_cuda_train_params_init": (None, [_P]),
    "nabo_cuda_radius_model_train": (_I, [_P, _P, _I, _I64, _I64, _I, _U, _D, _P, _P]),
    "nabo_cuda_radius_model_destroy": (_I, [_P]),
    "nabo_cuda_radius_model_predict_device": (_I, [_P, _P, _I, _I64, _I64, _D, _P, _P, _P]),
    "nabo_cuda_knn_learned_device": (_I, [_P, _P, _P, _I, _I64, _I64, _I, _D, _U, _D, _P, _P, _P, _P, _P]),
    "nabo_cuda_knn_learned": (_I, [_P, _P, _P, _I, _I64, _I64, _I, _D, _U, _D, _P, _P, _P, _P]),
    "nabo_cuda_radius_model_features_device": (_I, [_P, _P, _I, _I64, _I64, _P, _P]),
    "nabo_cuda_radius_model_gradients": (_I, [_P, _P, _P, _I64, _P, _P]),
    "nabo_cuda_radius_model_get": (_I, [_P, _P, _P]),
    "nabo_cuda_radius_model_set": (_I, [_P, _P, _P]),
    "nabo_cuda_batch_create": (_I, [_I, _I, _I, _P, _P, _I, _P]),
    "nabo_cuda_batch_destroy": (_I, [_P]),
    "nabo_cuda_batch_knn_radii_device": (_I, [_P, _P, _P, _D, _U, _D, _P, _P, _P, _P]),
    "nabo_cuda_batch_radius_model_train": (_I, [_P, _P, _P, _P, _P]),
    "nabo_cuda_batch_knn_learned_device": (_I, [_P, _P, _P, _D, _U, _D, _P, _P, _P, _P]),
    "nabo_cuda_batch_radius_model_predict_device": (_I, [_P, _P, _P, _D, _P, _P, _P]),
    "nabo_cuda_batch_radius_model_features_device": (_I, [_P, _P, _P, _P, _P]),
    "nabo_cuda_batch_set_queries": (_I, [_P, _P, _P]),
    "nabo_cuda_batch_build_device": (_I, [_P, _P, _P]),
    "nabo_cuda_batch_knn_device": (_I, [_P, _P, _D, _U, _D, _P, _P, _P]),
    "nabo_cuda_batch_run": (_I, [_P, _P, _P, _D, _U, _D, _P, _P, _P]),
    "nabo_cuda_batch_run_host": (_I, [_P, _P, _P, _D, _U, _D, _P, _P]),
    "nabo_cuda_batch_status": (_I, [_P, _P]),
    "nabo_cuda_batch_export_tree": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "nabo_cuda_get_info": (_I, [_P, _P]),
    "nabo_cuda_get_bounds": (_I, [_P, _P, _P]),
    "nabo_cuda_export_tree": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "nabo_cuda_profile": (_I, [_P, _I]),
    "nabo_cuda_last_kernel_ms": (_I, [_P, _P]),
    "nabo_cuda_last_error": (ctypes.c_char_p, []),
    "nabo_cuda_version": (ctypes.c_char_p, []),
    "nabo_cuda_measure_fma_peak": (_I, [_I, _P]),
}


class nabo_cuda_train_params(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("epochs", ctypes.c_int32),
        ("batch", ctypes.c_int32),
        ("lr", ctypes.c_float),
        ("safety", ctypes.c_float),
        ("targetMissRate", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("reserved", ctypes.c_int32 * 4),
    ]


class nabo_cuda_params(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("bucketSize", ctypes.c_uint32),
        ("queryOrdering", ctypes.c_int32),
        ("traversal", ctypes.c_int32),
        ("threadsPerBlock", ctypes.c_int32),
        ("pipelineChunks", ctypes.c_int32),
        ("splitRule", ctypes.c_int32),
        ("lanesPerQuery", ctypes.c_int32),
    ]


def _load() -> ctypes.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m libnabo_gb300.build` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_lib = None


def get() -> ctypes.CDLL:
    """The loaded library (loaded on first call)."""
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


class LazyLib:
    """Attribute access forwards to the library, loading it on first use."""

    def __getattr__(self, name):
        return getattr(get(), name)


lib = LazyLib()
