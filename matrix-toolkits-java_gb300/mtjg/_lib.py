"""ctypes binding of libmtjg.so (include/mtjg.h).

The shared library is built in-tree by ``matrix-toolkits-java_gb300/build.py``.
There is no fallback: if the library or a CUDA device is missing, loading or
creating a context raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(os.path.dirname(_HERE), "lib")
# MTJG_LIB points at another build of the library (e.g. one built with other
# tile settings); by default the in-tree build is loaded
LIB_PATH = os.environ.get("MTJG_LIB") or os.path.join(LIB_DIR, "libmtjg.so")
WORKLOADS_PATH = os.path.join(LIB_DIR, "libmtjg_workloads.so")

# status codes (include/mtjg.h)
OK = 0
NOT_CONVERGED_ITERATIONS = 1
NOT_CONVERGED_DIVERGENCE = 2
NOT_CONVERGED_BREAKDOWN = 3
ERR_ILLEGAL_ARGUMENT = 10
ERR_INDEX_OUT_OF_BOUNDS = 11
ERR_IO = 12
ERR_ZERO_PIVOT = 20
ERR_ZERO_DIAGONAL = 21
ERR_MISSING_DIAGONAL = 22
ERR_SINGULAR = 23
ERR_UNSUPPORTED = 30
ERR_CUDA = 40
ERR_OUT_OF_MEMORY = 41
ERR_DEVICE_TIMEOUT = 42

NORM_ONE, NORM_TWO, NORM_TWO_ROBUST, NORM_INFINITY = 0, 1, 2, 3
PC_IDENTITY, PC_JACOBI, PC_ILU, PC_ICC, PC_SSOR, PC_ILUT = 0, 1, 2, 3, 4, 5
CG, BICGSTAB, GMRES, BICG, CGS, QMR, CHEBYSHEV, IR = 0, 1, 2, 3, 4, 5, 6, 7
NUMERICS_FAST, NUMERICS_STRICT = 0, 1


class Monitor(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("rtol", C.c_double), ("atol", C.c_double),
                ("dtol", C.c_double), ("norm", C.c_int), ("history_cap", C.c_int)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("residual", C.c_double),
                ("detail", C.c_int), ("history_len", C.c_int), ("inner_iterations", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("max_systems", C.c_int), ("pool_rows", C.c_int64), ("max_iter", C.c_int),
                ("rtol", C.c_double), ("atol", C.c_double), ("dtol", C.c_double),
                ("inner_rtol", C.c_double), ("inner_max_iter", C.c_int), ("matrix_budget", C.c_int64)]


class ServerResult(C.Structure):
    _fields_ = [("ticket", C.c_int64), ("matrix", C.c_int), ("result", Result),
                ("latency_s", C.c_double), ("queue_s", C.c_double)]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64 = C.c_int64

# name -> (restype, argtypes)
PROTOTYPES = {
    "mtjg_last_error": (C.c_char_p, []),
    "mtjg_version": (C.c_char_p, []),
    "mtjg_monitor_defaults": (None, [C.POINTER(Monitor)]),
    "mtjg_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "mtjg_ctx_destroy": (C.c_int, [_vp]),
    "mtjg_ctx_set_numerics": (C.c_int, [_vp, C.c_int]),
    "mtjg_ctx_synchronize": (C.c_int, [_vp]),
    "mtjg_ctx_launch_count": (C.c_int64, [_vp]),
    "mtjg_ctx_event_record": (C.c_int, [_vp, C.c_int]),
    "mtjg_ctx_event_elapsed": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "mtjg_dev_alloc": (C.c_int, [_vp, _i64, C.POINTER(_vp)]),
    "mtjg_dev_free": (C.c_int, [_vp, _vp]),
    "mtjg_memcpy_h2d": (C.c_int, [_vp, _vp, _vp, _i64]),
    "mtjg_memcpy_d2h": (C.c_int, [_vp, _vp, _vp, _i64]),
    "mtjg_csr_upload": (C.c_int, [_vp, C.c_int, C.c_int, _ip, _ip, _dp, C.POINTER(_vp)]),
    "mtjg_csr_update_values": (C.c_int, [_vp, _dp]),
    "mtjg_csr_read_matrix_market": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp)]),
    "mtjg_csr_parse_matrix_market": (C.c_int, [_vp, C.c_char_p, _i64, C.POINTER(_vp)]),
    "mtjg_csr_parse_matrix_market_host": (C.c_int, [C.c_char_p, _i64, _ip, _ip, C.POINTER(_i64), _ip, _ip, _dp,
                                                    _i64]),
    "mtjg_vector_read_matrix_market": (C.c_int, [C.c_char_p, _dp, _i64, C.POINTER(_i64)]),
    "mtjg_vector_parse_matrix_market": (C.c_int, [C.c_char_p, _i64, _dp, _i64, C.POINTER(_i64)]),
    "mtjg_csr_to_host": (C.c_int, [_vp, _ip, _ip, _dp]),
    "mtjg_csr_upload_csc": (C.c_int, [_vp, C.c_int, C.c_int, _ip, _ip, _dp, C.POINTER(_vp)]),
    "mtjg_csr_upload_rows": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_i64), _ip, _ip, _dp, _i64,
                                       C.POINTER(_vp)]),
    "mtjg_csr_destroy": (C.c_int, [_vp]),
    "mtjg_csr_dims": (C.c_int, [_vp, _ip, _ip, C.POINTER(_i64)]),
    "mtjg_csr_mult": (C.c_int, [_vp, _dp, _dp]),
    "mtjg_csr_mult_add": (C.c_int, [_vp, C.c_double, _dp, _dp]),
    "mtjg_csr_trans_mult": (C.c_int, [_vp, _dp, _dp]),
    "mtjg_csr_trans_mult_add": (C.c_int, [_vp, C.c_double, _dp, _dp]),
    "mtjg_csr_mult_dev": (C.c_int, [_vp, _vp, _vp]),
    "mtjg_csr_mult_add_dev": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "mtjg_csr_trans_mult_dev": (C.c_int, [_vp, _vp, _vp]),
    "mtjg_csr_mult_add_norm_noalloc": (C.c_int, [_vp, C.c_double, _vp, _vp, _vp]),
    "mtjg_precond_create": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "mtjg_precond_set_matrix": (C.c_int, [_vp, _vp, _ip]),
    "mtjg_precond_apply": (C.c_int, [_vp, _dp, _dp]),
    "mtjg_precond_trans_apply": (C.c_int, [_vp, _dp, _dp]),
    "mtjg_precond_apply_dev": (C.c_int, [_vp, _vp, _vp]),
    "mtjg_precond_values": (C.c_int, [_vp, _dp, _i64, C.POINTER(_i64)]),
    "mtjg_precond_set_ssor": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double]),
    "mtjg_precond_set_ilut": (C.c_int, [_vp, C.c_double, C.c_int]),
    "mtjg_precond_pattern": (C.c_int, [_vp, _ip, _ip, _ip, _i64, C.POINTER(_i64)]),
    "mtjg_precond_destroy": (C.c_int, [_vp]),
    "mtjg_solver_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    "mtjg_solver_set_precond": (C.c_int, [_vp, _vp]),
    "mtjg_solver_set_monitor": (C.c_int, [_vp, C.POINTER(Monitor)]),
    "mtjg_solver_solve": (C.c_int, [_vp, _vp, _dp, _dp, C.POINTER(Result)]),
    "mtjg_solver_solve_dev": (C.c_int, [_vp, _vp, _vp, _vp, C.POINTER(Result)]),
    "mtjg_solver_history": (C.c_int, [_vp, _dp, _ip, C.c_int, _ip]),
    "mtjg_solver_destroy": (C.c_int, [_vp]),
    "mtjg_batch_upload": (C.c_int, [_vp, C.c_int, _ip, _ip, _ip, _dp, C.POINTER(_vp)]),
    "mtjg_solver_set_mixed": (C.c_int, [_vp, C.c_int, C.c_double, C.c_int]),
    "mtjg_solver_set_launch": (C.c_int, [_vp, C.c_int]),
    "mtjg_solver_set_matrix_monitor": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double]),
    "mtjg_solver_set_eigenvalues": (C.c_int, [_vp, C.c_double, C.c_double]),
    "mtjg_server_config_defaults": (None, [C.POINTER(ServerConfig)]),
    "mtjg_server_create": (C.c_int, [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "mtjg_server_add_matrix": (C.c_int, [_vp, C.c_int, _ip, _ip, _dp, _ip]),
    "mtjg_server_remove_matrix": (C.c_int, [_vp, C.c_int]),
    "mtjg_server_submit": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp, C.POINTER(C.c_int64)]),
    "mtjg_server_submit_solver": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, _dp, C.POINTER(C.c_int64)]),
    "mtjg_server_poll": (C.c_int, [_vp, C.POINTER(ServerResult), C.c_int, _ip]),
    "mtjg_server_drain": (C.c_int, [_vp, C.c_double]),
    "mtjg_server_stats": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_double)]),
    "mtjg_server_timing": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "mtjg_server_residency": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]),
    "mtjg_server_context": (C.c_int, [_vp, C.POINTER(_vp)]),
    "mtjg_server_destroy": (C.c_int, [_vp]),
    "mtjg_solver_batch_results": (C.c_int, [_vp, C.POINTER(Result), C.c_int]),
    "mtjg_batch_tuning": (C.c_int, [_i64, _i64, _ip]),
    "mtjg_solver_batch_history": (C.c_int, [_vp, C.c_int, _dp, _ip, C.c_int, _ip]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads libmtjg.so once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python matrix-toolkits-java_gb300/build.py)")
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().mtjg_last_error().decode(errors="replace")


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)
