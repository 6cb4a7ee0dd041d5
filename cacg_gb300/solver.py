"""Python mirror of the reference solver interface, over libcacg.so.

``cbcg_v1`` / ``bcbcg_v1`` take the same arguments with the same meaning as
the reference C functions (src/cbcgKernel.h:21, src/bcbcgKernel.h:22):
a block-row CSR (row_start, col_idx, csrdata), the RHS block B (n x m,
row-major), the solution block X (in/out), s, and the absolute threshold
epsilon on ||R(:,0)||; like the reference they return nothing, update X in
place and stop after 1000 (CBCG) / 100 (BCBCG) outer iterations.  The status
of the call is in ``last_status()`` instead of an exit().

``solve`` is the extended entry (cacg_solve): explicit Chebyshev bounds,
relative tolerance on every column's true residual, precision mode and
residual-replacement period.  All compute runs on the GPU through
libcacg.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

_KINDS = {"lap2d": 1, "lap3d7": 2, "st3d27": 3, "varcoef2d": 4}
_RHS = {"uniform": 0, "normal": 1, "beta25": 2, "ones": 3}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def gen_matrix(kind: str, N: int, shift: float = 0.0, sigma: float = 0.0, seed: int = 0):
    """Seeded CSR (int32 row_ptr, int32 col_idx, float64 val)."""
    lib = L.lib()
    k = _KINDS[kind]
    n = lib.cacg_gen_rows(k, N)
    nnz = lib.cacg_gen_nnz(k, N)
    rp = np.empty(n + 1, np.int32)
    ci = np.empty(nnz, np.int32)
    v = np.empty(nnz, np.float64)
    L.check(lib.cacg_gen_matrix(k, N, shift, sigma, seed, _ptr(rp), _ptr(ci), _ptr(v)),
            "cacg_gen_matrix")
    return rp, ci, v


def gen_rhs(dist: str, n: int, m: int, seed: int, a: float = 0.0, b: float = 1.0):
    out = np.empty((n, m), np.float64)
    L.check(L.lib().cacg_gen_rhs(_RHS[dist], n, m, seed, a, b, _ptr(out)), "cacg_gen_rhs")
    return out


@dataclass
class Params:
    s: int = 4
    bounds: object = "gerschgorin"  # "gerschgorin" | ("given", lo, hi) | ("lanczos", steps)
    tol: float = 1e-8
    tol_mode: str = "rel"           # "rel" (all columns, true residual) | "abs_col0"
    maxit: int = 1000
    precision: str = "fp64"         # "fp64" | "mixed"
    rr_period: int = 5
    gram: str = "auto"              # "auto" | "fma" | "dmma" | "tc" | "tc_slices" | "tc5"
    lanczos_seed: int = 12345
    stream: int = 0
    exact_updates: bool = False     # mixed: float-float X/R update products
    spmm_format: str = "auto"       # "auto" (DIA view when the matrix has one) | "csr"
                                    # | "dia_unstaged" (DIA without shared-memory staging)
    residual: str = "auto"          # mixed: "auto" (float-float replacements on DIA) | "fp64"
    use_graph: bool = False         # replay captured outer iterations (non-default stream)
    algorithm: str = "cacg"         # "cacg" (cbcg_v1 / bcbcg_v1) | "bcg" (block CG, FP64)

    def to_c(self) -> L.CacgParams:
        p = L.CacgParams()
        L.lib().cacg_params_default(C.byref(p))
        p.s = self.s
        b = self.bounds
        if b == "gerschgorin":
            p.bounds_mode = L.BOUNDS_GERSCHGORIN
        elif isinstance(b, tuple) and b[0] == "given":
            p.bounds_mode, p.lambda_min, p.lambda_max = L.BOUNDS_GIVEN, b[1], b[2]
        elif isinstance(b, tuple) and b[0] == "lanczos":
            p.bounds_mode, p.lanczos_steps = L.BOUNDS_LANCZOS, int(b[1])
        else:
            raise ValueError("bad bounds %r" % (b,))
        p.tol = self.tol
        p.tol_mode = {"rel": L.TOL_REL_ALL, "abs_col0": L.TOL_ABS_COL0}[self.tol_mode]
        p.maxit = self.maxit
        p.precision = {"fp64": L.FP64, "mixed": L.MIXED}[self.precision]
        p.rr_period = self.rr_period
        p.gram_variant = {"auto": L.GRAM_AUTO, "fma": L.GRAM_FMA, "dmma": L.GRAM_DMMA,
                          "tc": L.GRAM_TC, "tc_slices": L.GRAM_TC_SLICES,
                          "tc5": L.GRAM_TC5}[self.gram]
        p.lanczos_seed = self.lanczos_seed
        p.stream = self.stream or None
        p.exact_updates = 1 if self.exact_updates else 0
        p.spmm_format = {"auto": L.SPMM_AUTO, "csr": L.SPMM_CSR,
                         "dia_unstaged": L.SPMM_DIA_UNSTAGED}[self.spmm_format]
        p.residual_precision = {"auto": L.RESID_AUTO, "fp64": L.RESID_FP64}[self.residual]
        p.use_graph = 1 if self.use_graph else 0
        p.algorithm = {"cacg": L.ALG_CACG, "bcg": L.ALG_BCG}[self.algorithm]
        return p


def _result_dict(r: L.CacgResult, relres) -> dict:
    return {"status": r.status, "iterations": r.iterations,
            "residual_replacements": r.residual_replacements,
            "lambda_min": r.lambda_min, "lambda_max": r.lambda_max,
            "recurrence_norm0": r.recurrence_norm0, "true_relres_max": r.true_relres_max,
            "true_relres": relres, "seconds": r.seconds, "launches": r.launches}


def _csr(rp, ci, v):
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    v = np.ascontiguousarray(v, np.float64)
    A = L.CacgCsr(len(rp) - 1, len(v), _ptr(rp), _ptr(ci), _ptr(v))
    return A, (rp, ci, v)


def solve(rp, ci, v, B, X0=None, params: Params | None = None, overwrite_x0: bool = False,
          **kw):
    """Solve A X = B on the GPU (host arrays in and out).  Returns (X, info).

    overwrite_x0=True solves in place in X0 (a C-contiguous float64 n x m
    array, the reference's in/out X of cbcg_v1/bcbcg_v1): no host copy of the
    initial guess, the returned X is X0 itself."""
    params = params or Params(**kw)
    B = np.ascontiguousarray(B, np.float64)
    if B.ndim == 1:
        B = B[:, None]
    n, m = B.shape
    if overwrite_x0:
        if not (isinstance(X0, np.ndarray) and X0.dtype == np.float64 and X0.shape == (n, m)
                and X0.flags["C_CONTIGUOUS"] and X0.flags["WRITEABLE"]):
            raise ValueError("overwrite_x0 needs X0 as a writeable C-contiguous float64 "
                             "array of B's shape")
        X = X0
    else:
        X = np.zeros_like(B) if X0 is None else np.array(X0, np.float64, order="C", copy=True)
    A, keep = _csr(rp, ci, v)
    relres = np.zeros(m)
    res = L.CacgResult()
    res.true_relres = _ptr(relres)
    p = params.to_c()
    rc = L.lib().cacg_solve(C.byref(A), _ptr(B), _ptr(X), m, C.byref(p), C.byref(res))
    L.check(rc, "cacg_solve")
    return X, _result_dict(res, relres)


def _ref_structs(row_start, col_idx, csrdata, B, X):
    row_start = np.ascontiguousarray(row_start, np.int64)
    col_idx = np.ascontiguousarray(col_idx, np.int64)
    csrdata = np.ascontiguousarray(csrdata, np.float64)
    n = len(row_start) - 1
    mat = L.CsrTypeLocal(n, n, int(row_start[-1] - row_start[0]), 0, _ptr(row_start),
                         _ptr(col_idx), _ptr(csrdata))
    m = B.shape[1]
    Bd = L.DenseType(n, m, n, m, 0, _ptr(B))
    Xd = L.DenseType(n, m, n, m, 0, _ptr(X))
    return mat, Bd, Xd, (row_start, col_idx, csrdata)


def _dropin(fn, row_start, col_idx, csrdata, B, X, s, epsilon, myid, numprocs):
    if not (isinstance(X, np.ndarray) and X.dtype == np.float64 and X.flags.c_contiguous):
        raise TypeError("X must be a C-contiguous float64 array (updated in place)")
    B = np.ascontiguousarray(B, np.float64)
    if B.ndim == 1:
        B = B[:, None]
    Xv = X if X.ndim == 2 else X.reshape(-1, 1)
    mat, Bd, Xd, keep = _ref_structs(row_start, col_idx, csrdata, B, Xv)
    if s is None:  # bcg_v1 takes no s
        fn(mat, Bd, Xd, epsilon, myid, numprocs)
    else:
        fn(mat, Bd, Xd, s, epsilon, myid, numprocs)


def cbcg_v1(row_start, col_idx, csrdata, B, X, s, epsilon, myid=0, numprocs=1):
    """Drop-in for cbcg_v1 (src/cbcgKernel.h:21); X is updated in place."""
    _dropin(L.lib().cbcg_v1, row_start, col_idx, csrdata, B, X, s, epsilon, myid, numprocs)


def bcbcg_v1(row_start, col_idx, csrdata, B, X, s, epsilon, myid=0, numprocs=1):
    """Drop-in for bcbcg_v1 (src/bcbcgKernel.h:22); X is updated in place."""
    _dropin(L.lib().bcbcg_v1, row_start, col_idx, csrdata, B, X, s, epsilon, myid, numprocs)


def bcg_v1(row_start, col_idx, csrdata, B, X, epsilon, myid=0, numprocs=1):
    """Drop-in for bcg_v1, block CG (src/bcgKernel.h:22); X is updated in place."""
    _dropin(L.lib().bcg_v1, row_start, col_idx, csrdata, B, X, None, epsilon, myid, numprocs)


def last_status() -> int:
    return L.lib().cacg_last_status()


def last_iterations() -> int:
    return L.lib().cacg_last_iterations()


def set_dropin_maxit(maxit: int) -> None:
    L.lib().cacg_set_dropin_maxit(maxit)


def launch_count() -> int:
    return L.lib().cacg_launch_count()


class Matrix:
    """A CSR matrix resident on the device (cacg_matrix_*)."""

    def __init__(self, rp, ci, v, want_fp32=True):
        A, self._keep = _csr(rp, ci, v)
        self.n = A.n
        h = C.c_void_p()
        L.check(L.lib().cacg_matrix_create(C.byref(A), 1 if want_fp32 else 0, C.byref(h)),
                "cacg_matrix_create")
        self.h = h

    def device_bytes(self) -> int:
        return L.lib().cacg_matrix_device_bytes(self.h)

    def diagonals(self) -> int:
        """Diagonals of the DIA view (0: CSR only)."""
        return L.lib().cacg_matrix_diagonals(self.h)

    def solve_device(self, B_ptr: int, X_ptr: int, m: int, params: Params):
        """B_ptr / X_ptr: device addresses of n x m row-major float64 blocks."""
        relres = np.zeros(m)
        res = L.CacgResult()
        res.true_relres = _ptr(relres)
        p = params.to_c()
        rc = L.lib().cacg_solve_device(self.h, C.c_void_p(B_ptr), C.c_void_p(X_ptr), m,
                                       C.byref(p), C.byref(res))
        L.check(rc, "cacg_solve_device")
        return _result_dict(res, relres)

    def close(self):
        if self.h:
            L.lib().cacg_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching solve server (cacg_server_*)."""

    def __init__(self, mem_budget_bytes: int, max_active: int = 4, engine: str = "batched",
                 graphs: bool = True, batch_max_rows: int = 0):
        """engine: "batched" (one launch per phase over all admitted requests,
        steps replayed from CUDA graphs; requests above batch_max_rows rows,
        0 = 65536, -1 = no limit, take the per-request path) or "streams" (a
        stream and the single-request solver per request)."""
        cfg = L.CacgServerConfig(mem_budget_bytes, max_active,
                                 {"batched": 0, "streams": 1}[engine], 0 if graphs else 1,
                                 batch_max_rows)
        h = C.c_void_p()
        L.check(L.lib().cacg_server_create(C.byref(cfg), C.byref(h)), "cacg_server_create")
        self.h = h
        self._live = {}

    def submit(self, rp, ci, v, B, params: Params) -> int:
        A, keep = _csr(rp, ci, v)
        B = np.ascontiguousarray(B, np.float64)
        if B.ndim == 1:
            B = B[:, None]
        X = np.zeros_like(B)
        t = C.c_int64()
        p = params.to_c()
        L.check(L.lib().cacg_server_submit(self.h, C.byref(A), _ptr(B), B.shape[1], C.byref(p),
                                           _ptr(X), C.byref(t)), "cacg_server_submit")
        self._live[t.value] = (X, np.zeros(B.shape[1]))
        return t.value

    def _fetch(self, fn, ticket):
        X, relres = self._live[ticket]
        res = L.CacgResult()
        res.true_relres = _ptr(relres)
        rc = fn(self.h, ticket, C.byref(res))
        if rc == L.PENDING:
            return None
        self._live.pop(ticket)
        return X, _result_dict(res, relres)

    def poll(self, ticket):
        return self._fetch(L.lib().cacg_server_poll, ticket)

    def wait(self, ticket):
        return self._fetch(L.lib().cacg_server_wait, ticket)

    def stats(self):
        q, a, b = C.c_int64(), C.c_int64(), C.c_int64()
        L.lib().cacg_server_stats(self.h, C.byref(q), C.byref(a), C.byref(b))
        return {"queued": q.value, "active": a.value, "bytes_in_use": b.value}

    def engine_stats(self):
        steps, rep = C.c_int64(), C.c_int64()
        bps = (C.c_int32 * 8)()
        L.lib().cacg_server_engine_stats(self.h, C.byref(steps), C.byref(rep), bps, 8)
        kinds = ["spmm", "gram", "qupdate", "xrupdate"]
        return {"steps": steps.value, "graph_replays": rep.value,
                "blocks_per_sm": {"fp64": dict(zip(kinds, bps[:4])),
                                  "fp32": dict(zip(kinds, bps[4:]))}}

    def close(self):
        if self.h:
            L.lib().cacg_server_destroy(self.h)
            self.h = None
