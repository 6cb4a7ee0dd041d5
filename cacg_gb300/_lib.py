"""ctypes bindings of libcacg.so (the C ABI declared in include/cacg.h).

The library is built in-tree (cacg_gb300/libcacg.so) by cacg_gb300/build.py.
Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcacg.so")

# ---- status / enums (include/cacg.h) ----
OK, NOT_CONVERGED, PENDING = 0, 1, 2
ERR_ARG, ERR_OOM, ERR_CUDA, ERR_BREAKDOWN, ERR_TIMEOUT = -1, -2, -3, -4, -5
ERR_UNSUPPORTED, ERR_BUSY, ERR_NODEV = -6, -7, -8
BOUNDS_GERSCHGORIN, BOUNDS_GIVEN, BOUNDS_LANCZOS = 0, 1, 2
TOL_ABS_COL0, TOL_REL_ALL = 0, 1
FP64, MIXED = 0, 1
GRAM_AUTO, GRAM_FMA, GRAM_DMMA, GRAM_TC, GRAM_TC_SLICES, GRAM_TC5 = 0, 1, 2, 3, 4, 5
SPMM_AUTO, SPMM_CSR, SPMM_DIA_UNSTAGED = 0, 1, 2
ALG_CACG, ALG_BCG = 0, 1
RESID_AUTO, RESID_FP64 = 0, 1
VAL_F64, VAL_F32 = 0, 1
# or-ed into the vtype of the kernel entry points (cacg_k_qupdate / cacg_k_xrupdate)
XR_EXACT, VAL_TC5, VAL_TC5_CPASYNC, XR_FFSTATE = 16, 32, 64, 128


class CacgCsr(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("row_ptr", C.c_void_p),
                ("col_idx", C.c_void_p), ("val", C.c_void_p)]


class CacgParams(C.Structure):
    _fields_ = [("s", C.c_int32), ("bounds_mode", C.c_int32), ("lambda_min", C.c_double),
                ("lambda_max", C.c_double), ("lanczos_steps", C.c_int32),
                ("tol_mode", C.c_int32), ("tol", C.c_double), ("maxit", C.c_int32),
                ("precision", C.c_int32), ("rr_period", C.c_int32),
                ("gram_variant", C.c_int32), ("lanczos_seed", C.c_uint64),
                ("stream", C.c_void_p), ("use_graph", C.c_int32),
                ("exact_updates", C.c_int32), ("spmm_format", C.c_int32),
                ("residual_precision", C.c_int32), ("algorithm", C.c_int32),
                ("reserved", C.c_int32 * 3)]


class CacgResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_int32),
                ("residual_replacements", C.c_int32), ("m", C.c_int32),
                ("lambda_min", C.c_double), ("lambda_max", C.c_double),
                ("recurrence_norm0", C.c_double), ("true_relres_max", C.c_double),
                ("true_relres", C.c_void_p), ("seconds", C.c_double),
                ("launches", C.c_int64), ("reserved", C.c_int32 * 6)]


class CsrTypeLocal(C.Structure):  # src/DataTypes.h:22-41
    _fields_ = [("num_rows", C.c_long), ("num_cols", C.c_long), ("nnz", C.c_long),
                ("start", C.c_long), ("row_start", C.c_void_p), ("col_idx", C.c_void_p),
                ("csrdata", C.c_void_p)]


class DenseType(C.Structure):  # src/DataTypes.h:50-59
    _fields_ = [("local_num_row", C.c_long), ("local_num_col", C.c_long),
                ("global_num_row", C.c_long), ("global_num_col", C.c_long),
                ("start_idx", C.c_long), ("data", C.c_void_p)]


class CacgServerConfig(C.Structure):
    _fields_ = [("mem_budget_bytes", C.c_int64), ("max_active", C.c_int32),
                ("engine", C.c_int32), ("no_graphs", C.c_int32), ("batch_max_rows", C.c_int32),
                ("reserved", C.c_int32 * 4)]


_lib = None

_SIGS = {
    # drop-ins
    "cbcg_v1": (None, [CsrTypeLocal, DenseType, DenseType, C.c_long, C.c_double, C.c_int,
                       C.c_int]),
    "bcbcg_v1": (None, [CsrTypeLocal, DenseType, DenseType, C.c_long, C.c_double, C.c_int,
                        C.c_int]),
    "bcg_v1": (None, [CsrTypeLocal, DenseType, DenseType, C.c_double, C.c_int, C.c_int]),
    "cacg_last_status": (C.c_int, []),
    "cacg_last_iterations": (C.c_int, []),
    "cacg_set_dropin_maxit": (None, [C.c_int]),
    # extended
    "cacg_params_default": (None, [C.POINTER(CacgParams)]),
    "cacg_status_string": (C.c_char_p, [C.c_int]),
    "cacg_solve": (C.c_int, [C.POINTER(CacgCsr), C.c_void_p, C.c_void_p, C.c_int32,
                             C.POINTER(CacgParams), C.POINTER(CacgResult)]),
    "cacg_matrix_create": (C.c_int, [C.POINTER(CacgCsr), C.c_int32, C.POINTER(C.c_void_p)]),
    "cacg_matrix_destroy": (C.c_int, [C.c_void_p]),
    "cacg_matrix_device_bytes": (C.c_int64, [C.c_void_p]),
    "cacg_matrix_diagonals": (C.c_int32, [C.c_void_p]),
    "cacg_solve_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                    C.POINTER(CacgParams), C.POINTER(CacgResult)]),
    "cacg_workspace_bytes": (C.c_int64, [C.c_int64, C.c_int32, C.c_int32, C.c_int32]),
    # kernels
    "cacg_k_gerschgorin": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "cacg_k_spmm": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                              C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_double,
                              C.c_double, C.c_double, C.c_void_p]),
    "cacg_k_basis": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_double,
                               C.c_void_p, C.c_int64, C.c_void_p]),
    "cacg_k_gram": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_int64,
                              C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                              C.c_int64, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "cacg_k_gram_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_void_p, C.c_int64,
                                      C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                                      C.c_int64, C.c_int32, C.c_void_p, C.c_int32,
                                      C.c_void_p]),
    "cacg_set_pipeline_wait_limit": (C.c_int, [C.c_int64]),
    "cacg_k_qupdate": (C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "cacg_k_xrupdate": (C.c_int, [C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                                  C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "cacg_k_tsqr": (C.c_int, [C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p,
                              C.c_int64, C.c_void_p, C.c_void_p]),
    "cacg_k_lu": (C.c_int, [C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                            C.c_void_p, C.c_void_p]),
    # input files
    "cacg_read_mtx": (C.c_int, [C.c_char_p, C.POINTER(CsrTypeLocal)]),
    "cacg_csr_free": (None, [C.POINTER(CsrTypeLocal)]),
    "cacg_csr_row_block": (C.c_int, [C.POINTER(CsrTypeLocal), C.c_int, C.c_int,
                                     C.POINTER(CsrTypeLocal)]),
    "cacg_read_csv": (C.c_int, [C.c_char_p, C.c_int64, C.c_int64, C.c_void_p,
                                C.POINTER(C.c_int64)]),
    "cacg_dense_row_block": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_int,
                                       C.POINTER(DenseType)]),
    "cacg_dense_free": (None, [C.POINTER(DenseType)]),
    "cacg_launch_count": (C.c_int64, []),
    "cacg_profile_enable": (None, [C.c_int]),
    "cacg_profile_reset": (None, []),
    "cacg_profile_get": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "cacg_profile_calls": (C.c_int64, [C.c_int]),
    "cacg_profile_name": (C.c_char_p, [C.c_int]),
    # server
    "cacg_server_create": (C.c_int, [C.POINTER(CacgServerConfig), C.POINTER(C.c_void_p)]),
    "cacg_server_submit": (C.c_int, [C.c_void_p, C.POINTER(CacgCsr), C.c_void_p, C.c_int32,
                                     C.POINTER(CacgParams), C.c_void_p,
                                     C.POINTER(C.c_int64)]),
    "cacg_server_poll": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(CacgResult)]),
    "cacg_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(CacgResult)]),
    "cacg_server_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64)]),
    "cacg_server_engine_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                           C.c_int32]),
    "cacg_server_destroy": (C.c_int, [C.c_void_p]),
    # generators
    "cacg_gen_rows": (C.c_int64, [C.c_int, C.c_int64]),
    "cacg_gen_nnz": (C.c_int64, [C.c_int, C.c_int64]),
    "cacg_gen_matrix": (C.c_int, [C.c_int, C.c_int64, C.c_double, C.c_double, C.c_uint64,
                                  C.c_void_p, C.c_void_p, C.c_void_p]),
    "cacg_gen_rhs": (C.c_int, [C.c_int, C.c_int64, C.c_int, C.c_uint64, C.c_double,
                               C.c_double, C.c_void_p]),
    "cacg_det_log": (C.c_double, [C.c_double]),
    "cacg_det_exp": (C.c_double, [C.c_double]),
}


def lib():
    """Load libcacg.so (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libcacg.so is missing and could not be built")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def status_string(code: int) -> str:
    return lib().cacg_status_string(code).decode()


class CacgError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__("%s: %s (%d)" % (what or "cacg", status_string(code), code))
        self.code = code


def check(code: int, what: str = "") -> int:
    if code < 0:
        raise CacgError(code, what)
    return code
