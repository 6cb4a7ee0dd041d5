"""cacg_gb300 -- GB300 (sm_103a) implementation of the sclc/cacg
communication-avoiding Chebyshev-basis (block) CG hot path.

The compute lives in libcacg.so (hand-written CUDA, C ABI in include/cacg.h);
this package is a thin ctypes layer over it that mirrors the reference's
solver interface.
"""
from ._lib import CacgError, lib, status_string  # noqa: F401
from .io import csr_row_block, dense_row_block, read_csv, read_mtx  # noqa: F401
from .solver import (Matrix, Params, Server, bcbcg_v1, bcg_v1, cbcg_v1, gen_matrix, gen_rhs,  # noqa: F401
                     last_iterations, last_status, launch_count, set_dropin_maxit, solve)

__all__ = ["lib", "status_string", "CacgError", "Params", "solve", "cbcg_v1", "bcbcg_v1", "bcg_v1",
           "last_status", "last_iterations", "set_dropin_maxit", "launch_count", "Matrix",
           "Server", "gen_matrix", "gen_rhs", "read_mtx", "csr_row_block", "read_csv",
           "dense_row_block"]
