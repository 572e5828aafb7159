"""ctypes binding of libbola_gb300.so (declared in include/bola_gb300.h).

The library is loaded from bola_gb300/lib/ only; a missing library is an
error, never a silent fallback.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libbola_gb300.so")

_d = ctypes.c_double
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_c = ctypes.c_char
_p = ctypes.c_void_p
_int = ctypes.c_int

# name -> (restype, argtypes); mirrors include/bola_gb300.h
SIGNATURES = {
    "bola_version": (ctypes.c_char_p, []),
    "bola_last_error": (ctypes.c_char_p, []),
    "bola_set_simd_lanes": (_int, [_int]),
    "bola_get_simd_lanes": (_int, []),
    "bola_profile_enable": (_int, [_int]),
    "bola_profile_reset": (_int, []),
    "bola_profile_count": (_int, []),
    "bola_profile_read": (_int, [_int, ctypes.c_char_p, _int, _p, _p, _p, _p, _p]),
    "bola_measure_fp64_peak": (_int, [_p]),
    "bola_measure_dmma_peak": (_int, [_p]),
    "bola_measure_cluster_exchange": (_int, [_int, _int, _p]),
    "bola_selftest_bounded_waits": (_int, [_p, ctypes.c_uint32, _p]),
    "bola_idamax": (_int, [_i64, _p, _p, _p]),
    "bola_dscal": (_int, [_i64, _d, _p, _i64, _p]),
    "bola_dger": (_int, [_i64, _i64, _d, _p, _p, _i64, _p, _i64, _p]),
    "bola_ddot": (_int, [_i64, _p, _i64, _p, _i64, _p, _p]),
    "bola_daxpy": (_int, [_i64, _d, _p, _i64, _p, _i64, _p]),
    "bola_dlaswp": (_int, [_i64, _p, _i64, _i32, _i32, _p, _i32, _p]),
    "bola_dgemm": (_int, [_c, _c, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _d, _p, _i64, _p]),
    "bola_dgemm_noalloc": (_int, [_c, _c, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _d, _p, _i64, _p]),
    "bola_sgemm_tc_update": (_int, [_int, _i64, _i64, _p, _p, _p, _p, _p, _i64, _p, _p]),
    "bola_dgemm_oz_update": (_int, [_i64, _i64, _p, _p, _p, _i64, _p, _p]),
    "bola_sgetrf_mixed": (_int, [_int, _i64, _p, _i64, _p, _p, _p]),
    "bola_spotrf_mixed": (_int, [_int, _i64, _p, _i64, _p, _p]),
    "bola_dgemv_oz": (_int, [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p]),
    "bola_dtrsm": (_int, [_c, _c, _c, _c, _i64, _i64, _d, _p, _i64, _p, _i64, _p]),
    "bola_dsyrk": (_int, [_c, _c, _i64, _i64, _d, _p, _i64, _d, _p, _i64, _p]),
    "bola_dgetrf": (_int, [_i64, _i64, _p, _i64, _p, _p, _p]),
    "bola_dgetrf2": (_int, [_i64, _i64, _p, _i64, _p, _p, _p]),
    "bola_dpotrf": (_int, [_c, _i64, _p, _i64, _p, _p]),
    "bola_dpotrf2": (_int, [_c, _i64, _p, _i64, _p, _p]),
    "bola_dgetrs": (_int, [_i64, _i64, _p, _i64, _p, _p, _i64, _p]),
    "bola_dpotrs": (_int, [_c, _i64, _i64, _p, _i64, _p, _i64, _p]),
}



class MixedOpts(ctypes.Structure):
    _fields_ = [("factor_kind", ctypes.c_int), ("max_iterations", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("fallback_fp64", ctypes.c_int), ("gmres", ctypes.c_int), ("escalate", ctypes.c_int)]


class MixedInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("gmres_iterations", ctypes.c_int), ("path", ctypes.c_int),
                ("factor_info", ctypes.c_int), ("backward_error", ctypes.c_double),
                ("condition_estimate", ctypes.c_double), ("factorization", ctypes.c_int), ("reserved", ctypes.c_int)]


SIGNATURES["bola_dgesv_mixed"] = (_int, [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, ctypes.POINTER(MixedOpts),
                                         ctypes.POINTER(MixedInfo), _p])
SIGNATURES["bola_dposv_mixed"] = SIGNATURES["bola_dgesv_mixed"]



class BatchTuning(ctypes.Structure):
    """bola_batch_tuning (include/bola_gb300.h)."""
    _fields_ = [("group_size", ctypes.c_int32 * 8), ("panel_width", ctypes.c_int32 * 8),
                ("tile_rows", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class System(ctypes.Structure):
    """bola_system (include/bola_gb300.h)."""
    _fields_ = [("n", ctypes.c_int32), ("nrhs", ctypes.c_int32), ("kind", ctypes.c_int32), ("lda", ctypes.c_int32),
                ("ldb", ctypes.c_int32), ("reserved", ctypes.c_int32), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p)]


SIGNATURES.update({
    "bola_mixed_ctx_create": (_int, [_p]),
    "bola_mixed_ctx_destroy": (_int, [_p]),
    "bola_mixed_ctx_bytes": (_i64, [_p]),
    "bola_dgesv_mixed_ctx": (_int, [_p, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, ctypes.POINTER(MixedOpts),
                                    ctypes.POINTER(MixedInfo), _p]),
    "bola_dposv_mixed_ctx": (_int, [_p, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, ctypes.POINTER(MixedOpts),
                                    ctypes.POINTER(MixedInfo), _p]),
    "bola_batch_plan_create": (_int, [_i32, _p, _p, _p, _p]),
    "bola_batch_plan_create_tuned": (_int, [_i32, _p, _p, ctypes.POINTER(BatchTuning), _p]),
    "bola_batch_tuning_save": (_int, [ctypes.c_char_p, ctypes.POINTER(BatchTuning)]),
    "bola_batch_tuning_load": (_int, [ctypes.c_char_p, ctypes.POINTER(BatchTuning), _p]),
    "bola_batch_solve": (_int, [_p, _p, _p, _p]),
    "bola_batch_solve_graph": (_int, [_p, _p, _p, _p]),
    "bola_batch_plan_info": (_int, [_p, _p, _p, _p]),
    "bola_batch_plan_destroy": (_int, [_p]),
})



class ServerOpts(ctypes.Structure):
    """bola_server_opts (include/bola_gb300.h)."""
    _fields_ = [("slots", ctypes.c_int32), ("small_n", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("factor_kind", ctypes.c_int32), ("group_size", ctypes.c_int32 * 8),
                ("reserved", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("panel_width", ctypes.c_int32 * 8), ("tile_rows", ctypes.c_int32), ("reserved2", ctypes.c_int32)]



class RequestInfo(ctypes.Structure):
    """bola_request_info (include/bola_gb300.h)."""
    _fields_ = [("status", ctypes.c_int32), ("path", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("info", ctypes.c_int32), ("backward_error", ctypes.c_double), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("factorization", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


SIGNATURES.update({
    "bola_server_create": (_int, [ctypes.POINTER(ServerOpts), _p]),
    "bola_server_submit": (_int, [_p, _i64, _i64, _i32, _p, _p, _p]),
    "bola_server_wait": (_int, [_p, _i64, _p, ctypes.POINTER(RequestInfo)]),
    "bola_server_stats": (_int, [_p, _p, _p, _p]),
    "bola_server_destroy": (_int, [_p]),
})

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load():
    """Load (once) and return the CDLL with typed entry points."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryMissing(
            f"{LIB_PATH} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
