"""CPU oracles for the cacg_gb300 GPU path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package.  It wraps two shared libraries built by oracle/build.py:

* ``ref``  -- the reference sclc/cacg solver sources compiled as shipped
  (oracle/_ref/libcacgref.so), driven through oracle/ref_harness.c;
* ``port`` -- the project's C restatement (oracle/cacg_oracle.c), pinned
  bit-for-bit against ``ref`` by tests/test_oracle_pins.py.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_P = np.ctypeslib.ndpointer
_f64 = _P(dtype=np.float64, flags="C_CONTIGUOUS")
_i64 = _P(dtype=np.int64, flags="C_CONTIGUOUS")
_i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")

_ref = None
_port = None


def ref_available() -> bool:
    return ref_lib() is not None


def ref_lib():
    """oracle/_ref/libcacgref.so (built on demand), or None if the reference
    sources are neither present nor staged."""
    global _ref
    if _ref is None:
        path = _build.build_reference()
        if path is None:
            return None
        lib = C.CDLL(path)
        lib.cacg_ref_solve.restype = C.c_long
        lib.cacg_ref_solve.argtypes = [C.c_int, C.c_int, C.c_long, _i64, _i64, _f64, _f64,
                                       _f64, C.c_long, C.c_long, C.c_double, C.c_int,
                                       C.c_double, C.c_double, C.c_long, _f64, C.c_long,
                                       C.c_int, C.POINTER(C.c_double)]
        lib.cacg_ref_gerschgorin.argtypes = [C.c_long, _i64, _i64, _f64, _f64]
        lib.cacg_ref_basis.argtypes = [C.c_int, C.c_long, _i64, _i64, _f64, _f64, C.c_long,
                                       C.c_long, C.c_double, C.c_double, _f64]
        lib.cacg_ref_spmm.argtypes = [C.c_long, _i64, _i64, _f64, _f64, C.c_long, _f64]
        lib.cacg_ref_gram.argtypes = [C.c_int, C.c_long, _f64, C.c_long, _f64, C.c_long, _f64]
        lib.cacg_ref_tallsmall.argtypes = [C.c_long, _f64, C.c_long, _f64, C.c_long, _f64]
        lib.cacg_ref_lu.argtypes = [C.c_long, _f64, C.c_long, _f64, _f64]
        lib.cacg_ref_read_mtx.restype = C.c_long
        lib.cacg_ref_read_mtx.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_long),
                                          C.POINTER(C.c_long), C.POINTER(C.c_void_p),
                                          C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        lib.cacg_ref_free.argtypes = [C.c_void_p]
        lib.cacg_ref_parse_csv.argtypes = [C.c_char_p, C.c_long, C.c_long, _f64]
        _ref = lib
    return _ref


def port_lib():
    global _port
    if _port is None:
        lib = C.CDLL(_build.build_port())
        i64 = C.c_int64
        lib.or_gerschgorin.argtypes = [i64, _i32, _i32, _f64, _f64]
        lib.or_spmm.argtypes = [i64, _i32, _i32, _f64, _f64, i64, i64, _f64, i64]
        lib.or_basis.argtypes = [i64, _i32, _i32, _f64, _f64, i64, i64, C.c_double,
                                 C.c_double, _f64]
        lib.or_gram.argtypes = [i64, _f64, i64, _f64, i64, _f64]
        lib.or_tallsmall.argtypes = [i64, _f64, i64, _f64, i64, _f64]
        lib.or_lu.argtypes = [i64, _f64, i64, _f64, _f64]
        lib.or_solve.restype = i64
        lib.or_solve.argtypes = [i64, _i32, _i32, _f64, _f64, _f64, i64, i64, C.c_double,
                                 C.c_int, C.c_double, C.c_double, i64, _f64, i64]
        lib.or_true_relres.argtypes = [i64, _i32, _i32, _f64, _f64, _f64, i64, _f64]
        lib.cacg_gen_rows.restype = i64
        lib.cacg_gen_rows.argtypes = [C.c_int, i64]
        lib.cacg_gen_nnz.restype = i64
        lib.cacg_gen_nnz.argtypes = [C.c_int, i64]
        lib.cacg_gen_matrix.argtypes = [C.c_int, i64, C.c_double, C.c_double, C.c_uint64,
                                        _i32, _i32, _f64]
        lib.cacg_gen_rhs.argtypes = [C.c_int, i64, C.c_int, C.c_uint64, C.c_double,
                                     C.c_double, _f64]
        lib.cacg_det_log.restype = C.c_double
        lib.cacg_det_log.argtypes = [C.c_double]
        lib.cacg_det_exp.restype = C.c_double
        lib.cacg_det_exp.argtypes = [C.c_double]
        _port = lib
    return _port


# ------------------------------------------------------------------ inputs
KINDS = {"lap2d": 1, "lap3d7": 2, "st3d27": 3, "varcoef2d": 4}
RHS = {"uniform": 0, "normal": 1, "beta25": 2, "ones": 3}


def gen_matrix(kind: str, N: int, shift: float = 0.0, sigma: float = 0.0, seed: int = 0):
    """Seeded CSR (row_ptr int32, col_idx int32, val float64) from the shared
    generator cacg_gb300/csrc/cacg_gen.c."""
    lib = port_lib()
    k = KINDS[kind]
    n = lib.cacg_gen_rows(k, N)
    nnz = lib.cacg_gen_nnz(k, N)
    rp = np.empty(n + 1, np.int32)
    ci = np.empty(nnz, np.int32)
    v = np.empty(nnz, np.float64)
    if lib.cacg_gen_matrix(k, N, shift, sigma, seed, rp, ci, v) != 0:
        raise RuntimeError("generator failed")
    return rp, ci, v


def gen_rhs(dist: str, n: int, m: int, seed: int, a: float = 0.0, b: float = 1.0):
    out = np.empty(n * m, np.float64)
    if port_lib().cacg_gen_rhs(RHS[dist], n, m, seed, a, b, out) != 0:
        raise RuntimeError("rhs generator failed")
    return out.reshape(n, m)


# ------------------------------------------------------------ port wrappers
def port_spmm(rp, ci, v, X):
    X = np.ascontiguousarray(X, np.float64)
    n, w = X.shape
    Y = np.empty_like(X)
    port_lib().or_spmm(n, rp, ci, v, X, w, w, Y, w)
    return Y


def port_basis(rp, ci, v, R, s, alpha, beta):
    R = np.ascontiguousarray(R, np.float64)
    n, m = R.shape
    S = np.empty((n, s * m))
    port_lib().or_basis(n, rp, ci, v, R, m, s, alpha, beta, S)
    return S


def port_gram(L, R):
    L = np.ascontiguousarray(L, np.float64)
    R = np.ascontiguousarray(R, np.float64)
    Cm = np.empty((L.shape[1], R.shape[1]))
    port_lib().or_gram(L.shape[0], L, L.shape[1], R, R.shape[1], Cm)
    return Cm


def port_tallsmall(L, W):
    L = np.ascontiguousarray(L, np.float64)
    W = np.ascontiguousarray(W, np.float64)
    Y = np.empty((L.shape[0], W.shape[1]))
    port_lib().or_tallsmall(L.shape[0], L, L.shape[1], W, W.shape[1], Y)
    return Y


def port_lu(M, RHS_):
    M = np.ascontiguousarray(M, np.float64)
    RHS_ = np.ascontiguousarray(RHS_, np.float64)
    Y = np.empty_like(RHS_)
    port_lib().or_lu(M.shape[0], M, RHS_.shape[1], RHS_, Y)
    return Y


def port_gerschgorin(rp, ci, v):
    out = np.empty(2)
    port_lib().or_gerschgorin(len(rp) - 1, rp, ci, v, out)
    return out


def port_solve(rp, ci, v, B, X0, s, eps, bounds=None, maxit=100):
    """Returns (X, iterations, history of ||R(:,0)||)."""
    B = np.ascontiguousarray(B, np.float64)
    X = np.array(X0, np.float64, order="C", copy=True)
    n, m = B.shape
    hist = np.zeros(max(maxit, 1))
    mode, lo, hi = (0, 0.0, 0.0) if bounds is None else (1, bounds[0], bounds[1])
    it = port_lib().or_solve(n, rp, ci, v, B, X, m, s, eps, mode, lo, hi, maxit, hist,
                             len(hist))
    return X, int(it), hist[:it].copy()


def port_true_relres(rp, ci, v, B, X):
    B = np.ascontiguousarray(B, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    out = np.empty(B.shape[1])
    port_lib().or_true_relres(B.shape[0], rp, ci, v, B, X, B.shape[1], out)
    return out


# ------------------------------------------------------- reference wrappers
def _i64a(a):
    return np.ascontiguousarray(a, np.int64)


def ref_solve(rp, ci, v, B, X0, s, eps, bounds=None, maxit=100, nranks=1, quiet=True,
              algorithm="cacg"):
    """Run the reference cbcg_v1 (m == 1) / bcbcg_v1 (m > 1), or with
    algorithm="bcg" the block CG bcg_v1 (src/bcgKernel.c:22; s unused).
    Returns (X, iterations, history, seconds)."""
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference oracle unavailable")
    B = np.ascontiguousarray(B, np.float64)
    X = np.array(X0, np.float64, order="C", copy=True)
    n, m = B.shape
    hist = np.zeros(max(maxit, 1))
    secs = C.c_double(0.0)
    mode, lo, hi = (0, 0.0, 0.0) if bounds is None else (1, bounds[0], bounds[1])
    solver = 3 if algorithm == "bcg" else (1 if m == 1 else 2)
    it = lib.cacg_ref_solve(solver, nranks, n, _i64a(rp), _i64a(ci), v, B, X, m, s, eps,
                            mode, lo, hi, maxit, hist, len(hist), 1 if quiet else 0,
                            C.byref(secs))
    return X, int(it), hist[:it].copy(), secs.value


def ref_spmm(rp, ci, v, X):
    X = np.ascontiguousarray(X, np.float64)
    Y = np.empty_like(X)
    ref_lib().cacg_ref_spmm(X.shape[0], _i64a(rp), _i64a(ci), v, X, X.shape[1], Y)
    return Y


def ref_basis(rp, ci, v, R, s, alpha, beta, cbcg=False):
    R = np.ascontiguousarray(R, np.float64)
    n, m = R.shape
    S = np.zeros((n, s * m))
    ref_lib().cacg_ref_basis(1 if cbcg else 0, n, _i64a(rp), _i64a(ci), v, R, m, s, alpha,
                             beta, S)
    return S


def ref_gram(L, R, square=False):
    L = np.ascontiguousarray(L, np.float64)
    R = np.ascontiguousarray(R, np.float64)
    Cm = np.zeros((L.shape[1], R.shape[1]))
    ref_lib().cacg_ref_gram(1 if square else 0, L.shape[0], L, L.shape[1], R, R.shape[1], Cm)
    return Cm


def ref_tallsmall(L, W):
    L = np.ascontiguousarray(L, np.float64)
    W = np.ascontiguousarray(W, np.float64)
    Y = np.empty((L.shape[0], W.shape[1]))
    ref_lib().cacg_ref_tallsmall(L.shape[0], L, L.shape[1], W, W.shape[1], Y)
    return Y


def ref_lu(M, RHS_):
    M = np.ascontiguousarray(M, np.float64)
    RHS_ = np.ascontiguousarray(RHS_, np.float64)
    Y = np.zeros_like(RHS_)
    ref_lib().cacg_ref_lu(M.shape[0], M, RHS_.shape[1], RHS_, Y)
    return Y


def ref_gerschgorin(rp, ci, v):
    out = np.empty(2)
    ref_lib().cacg_ref_gerschgorin(len(rp) - 1, _i64a(rp), _i64a(ci), v, out)
    return out


def ref_read_mtx(path):
    """The reference's Matrix Market reader and COO -> CSR conversion
    (src/readMTX.c:8-135, src/matrixType.c:4-52): (row_start, col_idx, values,
    (num_rows, num_cols)).  Valid files only (the reference exits otherwise)."""
    lib = ref_lib()
    d, name = os.path.split(os.path.abspath(path))
    nr, nc = C.c_long(), C.c_long()
    prp, pci, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    nnz = lib.cacg_ref_read_mtx(os.fsencode(d + os.sep), os.fsencode(name), C.byref(nr),
                                C.byref(nc), C.byref(prp), C.byref(pci), C.byref(pv))
    try:
        rp = np.ctypeslib.as_array(C.cast(prp, C.POINTER(C.c_long)), (nr.value + 1,)).copy()
        ci = (np.ctypeslib.as_array(C.cast(pci, C.POINTER(C.c_long)), (nnz,)).copy()
              if nnz else np.zeros(0, np.int64))
        v = (np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_double)), (nnz,)).copy()
             if nnz else np.zeros(0))
    finally:
        for p in (prp, pci, pv):
            lib.cacg_ref_free(p)
    return rp.astype(np.int64), ci.astype(np.int64), v, (nr.value, nc.value)


def ref_parse_csv(path, rows, cols):
    """The reference's parseCSV (src/common.c:16-48)."""
    out = np.zeros((rows, cols))
    ref_lib().cacg_ref_parse_csv(os.fsencode(path), rows, cols, out)
    return out


def port_bcg(rp, ci, v, B, X0, eps, maxit=1000):
    """Numpy restatement of bcg_v1 (src/bcgKernel.c:22-462), FP64: returns
    (X, iterations, history of ||R(:,0)||).  Order of operations as in the
    reference: X += P alpha, then the test on the residual before this
    iteration's update (:311-424), then R -= AP alpha, beta and P (:427-457).
    The m x m solves use numpy's LAPACK solver, not the reference's no-pivot
    Crout LU (src/DLSsolvers.c:6-91): results agree to rounding."""
    rp = np.asarray(rp, np.int64)
    ci = np.asarray(ci, np.int64)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))

    def spmm(Xm):
        Y = np.zeros_like(Xm)
        np.add.at(Y, rows, v[:, None] * Xm[ci])
        return Y

    B = np.asarray(B, np.float64)
    X = np.array(X0, np.float64, copy=True)
    R = B - spmm(X)
    P = R.copy()
    G = R.T @ R
    hist = []
    it = 0
    for it in range(1, maxit + 1):
        AP = spmm(P)
        alpha = np.linalg.solve(P.T @ AP, G)
        X += P @ alpha
        rn = float(np.sqrt(R[:, 0] @ R[:, 0]))
        hist.append(rn)
        if rn < eps:
            break
        R -= AP @ alpha
        G2 = R.T @ R
        beta = np.linalg.solve(G, G2)
        P = R + P @ beta
        G = G2
    return X, it, np.array(hist)
