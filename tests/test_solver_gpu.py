"""Solver-level parity on the GPU.

FP64 mode vs the reference (oracle/_ref, or the pinned restatement): the
outer-iteration count within +-1 and the solution relative difference
<= 1e-6 (the contract's tolerance), on the same seeded matrices, RHS and
parameters.  Mixed mode: true relative residual <= tol on every column and
solution within 1e-6 of the FP64 solution.
"""
import numpy as np
import pytest

import cacg_gb300 as cg
import oracle as O

pytestmark = pytest.mark.gpu


def _ref(rp, ci, v, B, s, eps, bounds, maxit):
    if O.ref_available():
        X, it, hist, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), s, eps, bounds, maxit)
    else:
        X, it, hist = O.port_solve(rp, ci, v, B, np.zeros_like(B), s, eps, bounds, maxit)
    return X, it, hist


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_cbcg_config1_analytic_bounds(lib):
    """2-D 5-pt 128^2, U[0,1) seed 0, x0 = 0, s = 4, analytic bounds."""
    rp, ci, v = cg.gen_matrix("lap2d", 128)
    B = cg.gen_rhs("uniform", 16384, 1, 0)
    c = np.cos(np.pi / 129)
    bounds = (4 - 4 * c, 4 + 4 * c)
    eps = 1e-8 * np.linalg.norm(B[:, 0])
    Xr, itr, _ = _ref(rp, ci, v, B, 4, eps, bounds, 2000)
    X, info = cg.solve(rp, ci, v, B, s=4, bounds=("given",) + bounds, tol=eps,
                       tol_mode="abs_col0", maxit=2000)
    assert info["status"] == 0
    assert abs(info["iterations"] - itr) <= 1, (info["iterations"], itr)
    assert _rel(X, Xr) <= 1e-6
    assert info["true_relres_max"] <= 1e-8


def test_cbcg_dropin_config1(lib):
    """Drop-in cbcg_v1 (Gerschgorin bounds, reference semantics) vs reference."""
    rp, ci, v = cg.gen_matrix("lap2d", 128)
    B = cg.gen_rhs("uniform", 16384, 1, 0)
    eps = 1e-8 * np.linalg.norm(B[:, 0])
    Xr, itr, _ = _ref(rp, ci, v, B, 4, eps, None, 1000)
    X = np.zeros_like(B)
    cg.cbcg_v1(rp.astype(np.int64), ci.astype(np.int64), v, B, X, 4, eps)
    assert cg.last_status() == 0
    assert abs(cg.last_iterations() - itr) <= 1
    assert _rel(X, Xr) <= 1e-6


@pytest.mark.parametrize("kind,N,m,s,dist", [("lap3d7", 24, 8, 8, "normal"),
                                             ("st3d27", 16, 16, 6, "uniform"),
                                             ("lap2d", 48, 3, 5, "normal")])
def test_bcbcg_dropin_vs_reference(lib, kind, N, m, s, dist):
    rp, ci, v = cg.gen_matrix(kind, N)
    n = len(rp) - 1
    B = cg.gen_rhs(dist, n, m, 1, -1.0, 1.0)
    eps = 1e-8 * np.linalg.norm(B[:, 0])
    Xr, itr, _ = _ref(rp, ci, v, B, s, eps, None, 100)
    X = np.zeros_like(B)
    cg.bcbcg_v1(rp.astype(np.int64), ci.astype(np.int64), v, B, X, s, eps)
    assert cg.last_status() in (0, 1)
    assert abs(cg.last_iterations() - itr) <= 1
    assert _rel(X, Xr) <= 1e-6


def test_dropin_rejects_multirank(lib):
    rp, ci, v = cg.gen_matrix("lap2d", 8)
    B = np.ones((64, 1))
    X = np.zeros_like(B)
    cg.cbcg_v1(rp.astype(np.int64), ci.astype(np.int64), v, B, X, 4, 1e-8, myid=0, numprocs=2)
    assert cg.last_status() == -6


@pytest.mark.parametrize("gram", ["fma", "dmma"])
def test_fp64_rel_mode_all_columns(lib, gram):
    rp, ci, v = cg.gen_matrix("lap3d7", 20)
    n = len(rp) - 1
    B = cg.gen_rhs("normal", n, 8, 1)
    c = np.cos(np.pi / 21)
    X, info = cg.solve(rp, ci, v, B, s=8, bounds=("given", 6 - 6 * c, 6 + 6 * c), tol=1e-8,
                       maxit=200, gram=gram)
    assert info["status"] == 0
    assert info["true_relres_max"] <= 1e-8
    relres = O.port_true_relres(rp, ci, v, B, X)
    assert relres.max() <= 1e-8


def test_mixed_matches_fp64(lib):
    rp, ci, v = cg.gen_matrix("st3d27", 24)
    n = len(rp) - 1
    B = cg.gen_rhs("uniform", n, 16, 2, -1.0, 1.0)
    kw = dict(s=6, bounds=("given", 0.05, 52.0), tol=1e-8, maxit=300, rr_period=5)
    X64, i64 = cg.solve(rp, ci, v, B, precision="fp64", **kw)
    X32, i32 = cg.solve(rp, ci, v, B, precision="mixed", **kw)
    assert i64["status"] == 0 and i32["status"] == 0
    assert i32["true_relres_max"] <= 1e-8
    assert O.port_true_relres(rp, ci, v, B, X32).max() <= 1e-8
    assert _rel(X32, X64) <= 1e-6


def test_overwrite_x0_solves_in_place(lib):
    rp, ci, v = cg.gen_matrix("st3d27", 20)
    n = len(rp) - 1
    B = cg.gen_rhs("uniform", n, 8, 3, -1.0, 1.0)
    kw = dict(s=6, bounds=("given", 0.05, 52.0), tol=1e-8, maxit=300, rr_period=5,
              precision="mixed")
    X0 = np.full_like(B, 0.25)
    Xc, ic = cg.solve(rp, ci, v, B, X0, **kw)
    assert (X0 == 0.25).all()  # the copying path leaves X0 alone
    Xi, ii = cg.solve(rp, ci, v, B, X0, overwrite_x0=True, **kw)
    assert Xi is X0
    assert ic["iterations"] == ii["iterations"]
    assert np.array_equal(Xc, Xi)


def test_mtx_csv_inputs_through_dropin(lib):
    """The reference driver's input path (src/main.c: Matrix Market matrix,
    CSV right-hand sides): the library's readers feed the bcbcg_v1 drop-in;
    the oracle solves the same inputs.  The matrix rows are in file order
    (unsorted), so the CSR kernels run."""
    import os
    io = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")
    rp, ci, v, (n, nc) = cg.read_mtx(os.path.join(io, "lap2d_12_sym.mtx"))
    B, got = cg.read_csv(os.path.join(io, "rhs_144x4.csv"), n, 4)
    assert got == n and nc == n
    eps = 1e-8 * float(np.linalg.norm(B[:, 0]))
    X = np.zeros_like(B)
    cg.set_dropin_maxit(400)
    try:
        cg.bcbcg_v1(rp, ci, v, B, X, 4, eps)
        st, it = cg.last_status(), cg.last_iterations()
    finally:
        cg.set_dropin_maxit(0)
    assert st == 0
    Xo, ito, _ = _ref(rp, ci, v, B, 4, eps, None, 400)
    assert abs(it - ito) <= 1
    assert _rel(X, Xo) <= 1e-6


def test_mixed_lanczos_bounds_varcoef(lib):
    rp, ci, v = cg.gen_matrix("varcoef2d", 48, shift=1e-6, sigma=1.5, seed=3)
    n = len(rp) - 1
    B = cg.gen_rhs("beta25", n, 4, 3)
    X, info = cg.solve(rp, ci, v, B, s=4, bounds=("lanczos", 50), tol=1e-8, maxit=2000,
                       precision="mixed", rr_period=5)
    assert info["status"] == 0, info
    assert O.port_true_relres(rp, ci, v, B, X).max() <= 1e-8
    assert info["lambda_max"] > info["lambda_min"] > 0


def test_zero_rhs_column_reports_breakdown(lib):
    """A zero RHS column makes Q^T A Q singular (the reference would divide by
    zero silently); the solver reports CACG_ERR_BREAKDOWN instead."""
    rp, ci, v = cg.gen_matrix("lap2d", 16)
    B = cg.gen_rhs("normal", 256, 3, 1)
    B[:, 1] = 0.0
    with pytest.raises(cg.CacgError) as e:
        cg.solve(rp, ci, v, B, s=4, tol=1e-8, maxit=50)
    assert e.value.code == -4


def test_mixed_cuda_core_exact_variant(lib):
    """Mixed mode with the float-float Gram and X/R update (no tensor cores)."""
    rp, ci, v = cg.gen_matrix("st3d27", 20)
    n = len(rp) - 1
    B = cg.gen_rhs("uniform", n, 16, 2, -1.0, 1.0)
    X, info = cg.solve(rp, ci, v, B, s=6, bounds=("given", 0.05, 52.0), tol=1e-8, maxit=300,
                       precision="mixed", gram="fma", exact_updates=True)
    assert info["status"] == 0
    assert O.port_true_relres(rp, ci, v, B, X).max() <= 1e-8


@pytest.mark.parametrize("kind,N,m,s", [("lap3d7", 32, 8, 8), ("lap2d", 96, 4, 4),
                                        ("st3d27", 24, 5, 6)])
def test_mixed_tensor_core_converges_like_fp64(lib, kind, N, m, s):
    rp, ci, v = cg.gen_matrix(kind, N)
    n = len(rp) - 1
    B = cg.gen_rhs("normal", n, m, 7)
    kw = dict(s=s, bounds="gerschgorin", tol=1e-8, maxit=500)
    X64, i64 = cg.solve(rp, ci, v, B, precision="fp64", **kw)
    X32, i32 = cg.solve(rp, ci, v, B, precision="mixed", **kw)
    assert i32["status"] == 0 and i64["status"] == 0
    assert O.port_true_relres(rp, ci, v, B, X32).max() <= 1e-8
    assert i32["iterations"] <= i64["iterations"] + 3
