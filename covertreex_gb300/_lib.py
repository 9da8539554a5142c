"""ctypes binding of libcovertree_cuda.so (C ABI in include/covertree_cuda.h).

The library is built in-tree by ``covertreex_gb300._build``.  There is no CPU
fallback: if the shared object is missing or fails to load, every engine call
raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import _build

CT_OK = 0
CT_ERR_ARG = 1
CT_ERR_CUDA = 2
CT_ERR_STATE = 3
CT_ERR_UNSUPPORTED = 4
CT_ERR_TIMEOUT = 5
CT_ERR_NOMEM = 6

CT_KERNEL_RBF = 0
CT_KERNEL_MATERN52 = 1
CT_ORDER_NATURAL = 0
CT_ORDER_HILBERT = 1
CT_ORDER_MORTON = 2
CT_FORM_DENSE = 0
CT_FORM_TREE = 1
CT_FORM_SCREENED = 2
CT_BUILD_METRIC_ONLY = 1
CT_BUILD_QUERY_SLAB = 2
CT_NOALLOC_SCRATCH_BYTES = 64 << 20

FORMS = {"dense": CT_FORM_DENSE, "tree": CT_FORM_TREE, "screened": CT_FORM_SCREENED}

#: every symbol include/covertree_cuda.h declares
EXPORTED_SYMBOLS = (
    "ct_version",
    "ct_set_timing",
    "ct_set_cta_budget",
    "ct_last_error",
    "ct_build_residual",
    "ct_knn_residual",
    "ct_knn_euclidean",
    "ct_knn_residual_dense_noalloc",
    "ct_tree_arrays",
    "ct_tree_shape",
    "ct_debug_screen_dots",
    "ct_free",
    "ct_vfactor_create",
    "ct_vfactor_embed",
    "ct_vfactor_chol",
    "ct_vfactor_free",
    "ct_knn_residual_points",
    "ct_prepare_screened",
    "ct_tree_inputs",
    "ct_tree_device_bytes",
    "ct_batch_create",
    "ct_batch_clear",
    "ct_batch_add_ids",
    "ct_batch_add_points",
    "ct_batch_set_shape",
    "ct_batch_autotune",
    "ct_batch_run",
    "ct_batch_get_shape",
    "ct_batch_reserve",
    "ct_batch_free",
    "ct_batch_order",
    "ct_luby_mis",
    "ct_tree_build_info",
    "ct_tree_extend",
    "ct_tree_subset",
)


class CtStats(ctypes.Structure):
    _fields_ = [
        ("distance_evals", ctypes.c_int64),
        ("pairs_screened", ctypes.c_int64),
        ("pairs_rescored", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("device_ms", ctypes.c_double),
        ("screen_ms", ctypes.c_double),
        ("threshold_ms", ctypes.c_double),
        ("rescore_ms", ctypes.c_double),
        ("screen_pairs_main", ctypes.c_int64),
        ("overflow_queries", ctypes.c_int64),
        ("pairs_exhaustive", ctypes.c_int64),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class EngineError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[ct error {code}] {message}")
        self.code = code


_lock = threading.Lock()
_handle = None


def library_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the configured ctypes CDLL."""
    global _handle
    with _lock:
        if _handle is not None:
            return _handle
        path = _build.LIB_PATH
        if build_if_missing and _build.needs_build():
            _build.build_library()
        if not path.exists():
            raise RuntimeError(f"libcovertree_cuda.so not found at {path}; run covertreex_gb300._build.build_library()")
        L = ctypes.CDLL(str(path))
        vp = ctypes.c_void_p
        i64, i32, f32, u64 = ctypes.c_int64, ctypes.c_int32, ctypes.c_float, ctypes.c_uint64
        L.ct_version.restype = ctypes.c_int
        L.ct_version.argtypes = []
        L.ct_set_timing.restype = ctypes.c_int
        L.ct_set_timing.argtypes = [ctypes.c_int]
        L.ct_set_cta_budget.restype = ctypes.c_int
        L.ct_set_cta_budget.argtypes = [ctypes.c_int32]
        L.ct_last_error.restype = ctypes.c_char_p
        L.ct_last_error.argtypes = []
        L.ct_build_residual.restype = ctypes.c_int
        L.ct_build_residual.argtypes = [vp, vp, vp, i64, i32, i32, f32, ctypes.POINTER(ctypes.c_float), i32, i32,
                                        i32, i32, u64, i32, vp, ctypes.POINTER(vp)]
        L.ct_tree_subset.restype = ctypes.c_int
        L.ct_tree_subset.argtypes = [vp, vp, i64, vp, ctypes.POINTER(vp)]
        L.ct_tree_extend.restype = ctypes.c_int
        L.ct_tree_extend.argtypes = [vp, vp, vp, vp, i64, vp, ctypes.POINTER(vp)]
        L.ct_knn_residual.restype = ctypes.c_int
        L.ct_knn_residual.argtypes = [vp, vp, i64, i32, i32, i32, vp, vp, ctypes.POINTER(CtStats), vp]
        L.ct_knn_euclidean.restype = ctypes.c_int
        L.ct_knn_euclidean.argtypes = [vp, i64, i32, vp, i64, i32, i32, vp, vp, vp]
        L.ct_knn_residual_dense_noalloc.restype = ctypes.c_int
        L.ct_knn_residual_dense_noalloc.argtypes = [vp, vp, vp, i64, i32, i32, f32, ctypes.POINTER(ctypes.c_float),
                                                    i32, i32, vp, i64, i32, i32, vp, vp, vp]
        L.ct_tree_arrays.restype = ctypes.c_int
        L.ct_tree_arrays.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.ct_tree_shape.restype = ctypes.c_int
        L.ct_tree_shape.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i32), ctypes.POINTER(i32)]
        L.ct_debug_screen_dots.restype = ctypes.c_int
        L.ct_debug_screen_dots.argtypes = [vp, vp, vp, vp, vp]
        L.ct_free.restype = ctypes.c_int
        L.ct_free.argtypes = [vp]
        f64 = ctypes.c_double
        L.ct_vfactor_create.restype = ctypes.c_int
        L.ct_vfactor_create.argtypes = [vp, i32, i32, i32, f64, f64, vp, ctypes.POINTER(vp)]
        L.ct_vfactor_embed.restype = ctypes.c_int
        L.ct_vfactor_embed.argtypes = [vp, vp, i64, vp, vp, vp]
        L.ct_vfactor_chol.restype = ctypes.c_int
        L.ct_vfactor_chol.argtypes = [vp, vp, vp]
        L.ct_vfactor_free.restype = ctypes.c_int
        L.ct_vfactor_free.argtypes = [vp]
        ip32 = ctypes.POINTER(i32)
        L.ct_tree_inputs.restype = ctypes.c_int
        L.ct_tree_inputs.argtypes = [vp, vp, vp, vp, vp]
        L.ct_prepare_screened.restype = ctypes.c_int
        L.ct_prepare_screened.argtypes = [vp, vp]
        L.ct_tree_device_bytes.restype = ctypes.c_int
        L.ct_tree_device_bytes.argtypes = [vp, ctypes.POINTER(i64)]
        L.ct_knn_residual_points.restype = ctypes.c_int
        L.ct_knn_residual_points.argtypes = [vp, vp, vp, vp, i64, i32, i32, vp, vp, ctypes.POINTER(CtStats), vp]
        L.ct_batch_create.restype = ctypes.c_int
        L.ct_batch_create.argtypes = [ctypes.POINTER(vp)]
        L.ct_batch_clear.restype = ctypes.c_int
        L.ct_batch_clear.argtypes = [vp]
        L.ct_batch_add_ids.restype = ctypes.c_int
        L.ct_batch_add_ids.argtypes = [vp, vp, vp, i64, i32, i32, vp, vp]
        L.ct_batch_add_points.restype = ctypes.c_int
        L.ct_batch_add_points.argtypes = [vp, vp, vp, vp, vp, i64, i32, vp, vp]
        L.ct_batch_set_shape.restype = ctypes.c_int
        L.ct_batch_set_shape.argtypes = [vp, i32, i32, i32]
        L.ct_batch_autotune.restype = ctypes.c_int
        L.ct_batch_autotune.argtypes = [vp, i32, vp, ip32, ip32, ip32]
        L.ct_batch_run.restype = ctypes.c_int
        L.ct_batch_run.argtypes = [vp, i32, ctypes.POINTER(CtStats), vp]
        L.ct_batch_get_shape.restype = ctypes.c_int
        L.ct_batch_get_shape.argtypes = [vp, ip32, ip32, ip32, ip32, ctypes.POINTER(i64)]
        L.ct_batch_reserve.restype = ctypes.c_int
        L.ct_batch_reserve.argtypes = [vp, i32, i32, i32]
        L.ct_batch_free.restype = ctypes.c_int
        L.ct_batch_free.argtypes = [vp]
        L.ct_batch_order.restype = ctypes.c_int
        L.ct_batch_order.argtypes = [vp, i64, i32, i32, vp, vp]
        L.ct_tree_build_info.restype = ctypes.c_int
        L.ct_tree_build_info.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(i64),
                                         ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_double)]
        L.ct_luby_mis.restype = ctypes.c_int
        L.ct_luby_mis.argtypes = [vp, vp, i64, u64, vp, ip32, vp]
        _handle = L
        return L


def check(rc: int) -> None:
    if rc != CT_OK:
        msg = load().ct_last_error()
        raise EngineError(rc, msg.decode() if msg else "")
