"""The reference's file inputs (host side, libcacg.so):

* ``read_mtx``       -- Matrix Market matrix -> CSR (src/readMTX.c:8-135 and
                        src/matrixType.c:4-52: symmetric files mirrored, each
                        row's entries in file order, 0-based int64 indices);
* ``csr_row_block``  -- rank ``myid``'s block of rows
                        (src/SparseMatrixDistribution.c:7-205);
* ``read_csv``       -- comma-separated right-hand sides (src/common.c:16-48);
* ``dense_row_block``-- rank ``myid``'s block of RHS rows (src/GetRHS.c:124-208).

Errors raise CacgError (the reference calls exit() or assert()).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L


def _take_csr(m: L.CsrTypeLocal):
    """Copy a library-allocated csrType_local into numpy arrays and free it."""
    try:
        n, nnz = m.num_rows, m.nnz
        rp = np.ctypeslib.as_array(C.cast(m.row_start, C.POINTER(C.c_long)), (n + 1,)).copy()
        if nnz > 0:
            ci = np.ctypeslib.as_array(C.cast(m.col_idx, C.POINTER(C.c_long)), (nnz,)).copy()
            v = np.ctypeslib.as_array(C.cast(m.csrdata, C.POINTER(C.c_double)), (nnz,)).copy()
        else:
            ci, v = np.zeros(0, np.int64), np.zeros(0, np.float64)
        return rp.astype(np.int64), ci.astype(np.int64), v, m.num_cols, m.start
    finally:
        L.lib().cacg_csr_free(C.byref(m))


def read_mtx(path: str):
    """(row_start, col_idx, values, (num_rows, num_cols)) of a Matrix Market
    coordinate file; int64 indices, FP64 values."""
    m = L.CsrTypeLocal()
    L.check(L.lib().cacg_read_mtx(os.fsencode(path), C.byref(m)), "cacg_read_mtx")
    rp, ci, v, ncols, _ = _take_csr(m)
    return rp, ci, v, (len(rp) - 1, ncols)


def csr_row_block(row_start, col_idx, csrdata, num_cols: int, myid: int, numprocs: int):
    """Rank ``myid``'s rows: (row_start rebased to 0, global col_idx, values,
    start row)."""
    rp = np.ascontiguousarray(row_start, np.int64)
    ci = np.ascontiguousarray(col_idx, np.int64)
    v = np.ascontiguousarray(csrdata, np.float64)
    g = L.CsrTypeLocal(len(rp) - 1, num_cols, len(v), 0, rp.ctypes.data, ci.ctypes.data,
                       v.ctypes.data)
    out = L.CsrTypeLocal()
    L.check(L.lib().cacg_csr_row_block(C.byref(g), myid, numprocs, C.byref(out)),
            "cacg_csr_row_block")
    lrp, lci, lv, _, start = _take_csr(out)
    return lrp, lci, lv, start


def read_csv(path: str, rows: int, cols: int):
    """(rows x cols FP64 array, rows actually read); missing rows stay zero."""
    out = np.zeros((rows, cols), np.float64)
    got = C.c_int64(0)
    L.check(L.lib().cacg_read_csv(os.fsencode(path), rows, cols, out.ctypes.data,
                                  C.byref(got)), "cacg_read_csv")
    return out, got.value


def dense_row_block(a, myid: int, numprocs: int):
    """Rank ``myid``'s block of rows of a (rows x cols) array: (block, fields
    of the reference's denseType)."""
    a = np.ascontiguousarray(a, np.float64)
    if a.ndim == 1:
        a = a[:, None]
    d = L.DenseType()
    L.check(L.lib().cacg_dense_row_block(a.ctypes.data, a.shape[0], a.shape[1], myid, numprocs,
                                         C.byref(d)), "cacg_dense_row_block")
    try:
        blk = np.ctypeslib.as_array(C.cast(d.data, C.POINTER(C.c_double)),
                                    (d.local_num_row * d.local_num_col,)).copy() \
            if d.local_num_row * d.local_num_col > 0 else np.zeros(0)
        fields = {f: getattr(d, f) for f in ("local_num_row", "local_num_col", "global_num_row",
                                             "global_num_col", "start_idx")}
        return blk.reshape(d.local_num_row, d.local_num_col), fields
    finally:
        L.lib().cacg_dense_free(C.byref(d))
