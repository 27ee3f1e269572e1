"""ctypes binding of libcelllist_cuda.so (the C ABI in include/celllistmap_gb300.h).

This is the product's only path to the GPU: there is no CPU fallback.  If the
library is missing or cannot create a CUDA stream, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcelllist_cuda.so")

# enums (include/celllistmap_gb300.h)
CLM_F32, CLM_F64 = 0, 1
CLM_ORTHO, CLM_TRICLINIC, CLM_NONPERIODIC = 0, 1, 2
CLM_PREC_EXACT, CLM_PREC_SPLIT = 0, 1
OP = {
    "nl": 1, "count": 2, "sum_d2": 3, "sum_d": 4, "sum_inv_d": 5, "soft_energy": 6, "soft_forces": 7,
    "lj_energy": 8, "lj_forces": 9, "mindist": 10, "rhist": 11, "inv_d_forces": 12, "lj_adjoint": 13,
    "weighted_inv_d": 14,
}
STATUS = {
    0: "CLM_OK", 1: "CLM_ERR_ARG", 2: "CLM_ERR_CELL_TOO_SMALL", 3: "CLM_ERR_NAN", 4: "CLM_ERR_DIM",
    5: "CLM_ERR_CUDA", 6: "CLM_ERR_CAPACITY", 7: "CLM_ERR_STATE", 8: "CLM_ERR_TIMEOUT", 9: "CLM_ERR_NOMEM",
    10: "CLM_ERR_LCELL", 11: "CLM_ERR_NONPERIODIC_CELL", 12: "CLM_ERR_INTERNAL",
}

# Every symbol declared in include/celllistmap_gb300.h
EXPORTS = [
    "clm_create", "clm_destroy", "clm_set_stream", "clm_set_box", "clm_set_positions", "clm_build",
    "clm_set_precision", "clm_run", "clm_run_noalloc", "clm_nl_count", "clm_nl_fetch", "clm_get_box", "clm_get_celllist_info",
    "clm_fetch_celllist", "clm_last_timings", "clm_lj_adjoint", "clm_batched_create", "clm_batched_set_systems",
    "clm_batched_run", "clm_batched_status", "clm_batched_set_graph", "clm_batched_set_config",
    "clm_batched_autotune", "clm_batched_last_step", "clm_stats", "clm_device_allocations", "clm_last_error",
    "clm_version",
]


class OpParams(C.Structure):
    _fields_ = [("p", C.c_double * 8), ("ntypes", C.c_int32), ("nbins", C.c_int32), ("types_x", C.c_void_p),
                ("types_y", C.c_void_p), ("eps_table", C.c_void_p), ("sig_table", C.c_void_p),
                ("vel_x", C.c_void_p), ("vel_y", C.c_void_p), ("bins", C.c_void_p),
                ("params_on_device", C.c_int32), ("reserved", C.c_int32),
                ("weights_x", C.c_void_p), ("weights_y", C.c_void_p)]


class Outputs(C.Structure):
    _fields_ = [("scalar", C.c_double), ("count", C.c_int64), ("min_i", C.c_int64), ("min_j", C.c_int64),
                ("min_d", C.c_double), ("forces_x", C.c_void_p), ("forces_y", C.c_void_p),
                ("hist_count", C.c_void_p), ("hist_sum", C.c_void_p), ("out_on_device", C.c_int32),
                ("index_base", C.c_int32), ("adjoint", C.c_void_p)]


class BatchOutputs(C.Structure):
    _fields_ = [("scalar", C.c_void_p), ("count", C.c_void_p), ("forces", C.c_void_p), ("out_on_device", C.c_int32),
                ("reserved", C.c_int32)]


_lib = None
_lock = threading.Lock()


def _declare(L):
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    L.clm_create.argtypes = [i32, i32, i32, C.POINTER(vp)]
    L.clm_destroy.argtypes = [vp]
    L.clm_set_stream.argtypes = [vp, vp]
    L.clm_set_box.argtypes = [vp, dp, i32, C.c_double, i32]
    L.clm_set_positions.argtypes = [vp, i32, vp, i64, i32]
    L.clm_build.argtypes = [vp]
    L.clm_set_precision.argtypes = [vp, i32]
    L.clm_run.argtypes = [vp, i32, C.POINTER(OpParams), C.POINTER(Outputs)]
    L.clm_run_noalloc.argtypes = [vp, i32, C.POINTER(OpParams), C.POINTER(Outputs)]
    L.clm_nl_count.argtypes = [vp, C.POINTER(i64)]
    L.clm_nl_fetch.argtypes = [vp, vp, vp, vp, i64, i32, i32]
    L.clm_get_box.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.clm_get_celllist_info.argtypes = [vp, i32, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]
    L.clm_fetch_celllist.argtypes = [vp, i32, i64, vp, vp, vp, vp, i32]
    L.clm_last_timings.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.clm_lj_adjoint.argtypes = [vp, C.POINTER(OpParams), C.POINTER(Outputs)]
    L.clm_batched_create.argtypes = [i32, i32, C.POINTER(vp)]
    L.clm_batched_set_systems.argtypes = [vp, i64, vp, vp, i32, C.c_double, i32]
    L.clm_batched_run.argtypes = [vp, i32, vp, vp, vp]
    L.clm_batched_status.argtypes = [vp, vp, i64]
    L.clm_batched_set_graph.argtypes = [vp, i32]
    L.clm_batched_set_config.argtypes = [vp, i32, i32, i32]
    L.clm_batched_autotune.argtypes = [vp, i32, vp, vp, i32, vp, C.POINTER(C.c_float)]
    L.clm_batched_last_step.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(i64)]
    L.clm_stats.argtypes = [vp, C.POINTER(i64)]
    L.clm_device_allocations.argtypes = [C.POINTER(i64), C.POINTER(i64)]
    L.clm_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    for name in EXPORTS:
        if name != "clm_version":
            getattr(L, name).restype = i32
    L.clm_version.restype = C.c_char_p
    L.clm_version.argtypes = []


def load(path: str | None = None):
    """Load the CUDA library (raises if it was not built: there is no fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise ImportError(f"libcelllist_cuda.so not found at {p}; build it with "
                                  "celllistmap.jl_gb300/build_lib.py (nvcc, sm_103a)")
            L = C.CDLL(p)
            _declare(L)
            _lib = L
    return _lib


def lib_path() -> str:
    return LIB_PATH
