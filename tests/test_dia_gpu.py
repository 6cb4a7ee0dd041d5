"""DIA view of stencil matrices: the solver over the DIA SpMM gives results
bit-identical to the CSR block kernels (same FMA order per row; one column
agrees up to rounding), and matrices that are not diagonal-structured stay
CSR-only."""
import numpy as np
import pytest
import torch

import cacg_gb300 as cg

pytestmark = pytest.mark.gpu


def _solve_dev(M, B, p):
    dB = torch.from_numpy(B).cuda()
    dX = torch.zeros_like(dB)
    info = M.solve_device(dB.data_ptr(), dX.data_ptr(), B.shape[1], p)
    torch.cuda.synchronize()
    return dX.cpu().numpy(), info


@pytest.mark.parametrize("kind,N,ndiag,m,s", [("lap2d", 40, 5, 3, 4), ("lap3d7", 14, 7, 8, 6),
                                              ("st3d27", 12, 27, 16, 6), ("varcoef2d", 30, 5, 4, 4),
                                              ("lap2d", 33, 5, 1, 4)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_dia_solve_bit_identical_to_csr(lib, kind, N, ndiag, m, s, prec):
    rp, ci, v = cg.gen_matrix(kind, N, shift=1e-3, sigma=1.0, seed=5)
    n = len(rp) - 1
    B = cg.gen_rhs("normal", n, m, 3)
    M = cg.Matrix(rp, ci, v, want_fp32=True)
    assert M.diagonals() == ndiag
    # FP64 residual replacements on both paths (the float-float replacement
    # exists only over the DIA view)
    kw = dict(s=s, bounds="gerschgorin", tol=1e-8, maxit=400, precision=prec, residual="fp64")
    Xd, idia = _solve_dev(M, B, cg.Params(spmm_format="auto", **kw))
    Xc, icsr = _solve_dev(M, B, cg.Params(spmm_format="csr", **kw))
    M.close()
    assert idia["status"] == 0 and icsr["status"] == 0
    if m == 1:
        # one column: the CSR SpMV splits a row over lanes (shuffle reduction),
        # the DIA kernel sums the row in column order -- both converge, and
        # the solutions agree within the solution tolerance of the parity tests
        assert abs(idia["iterations"] - icsr["iterations"]) <= 1
        assert idia["true_relres_max"] <= 1e-8 and icsr["true_relres_max"] <= 1e-8
        assert np.linalg.norm(Xd - Xc) <= 1e-6 * np.linalg.norm(Xc)
    else:
        assert idia["iterations"] == icsr["iterations"]
        assert np.array_equal(Xd, Xc)


@pytest.mark.parametrize("kind,N,m,s", [("st3d27", 40, 16, 6), ("st3d27", 26, 32, 3),
                                        ("lap3d7", 48, 16, 4), ("lap2d", 300, 16, 4),
                                        ("st3d27", 20, 20, 4), ("st3d27", 12, 16, 6)])
def test_staged_dia_bit_identical(lib, kind, N, m, s):
    """MIXED, 16k-column blocks: the shared-memory staged DIA SpMM (bands of
    diagonals in TMA-fed rings; three bands for the 3-D grids and the 300^2
    grid, one for 12^3) against the unstaged DIA kernel and CSR; m = 20 is
    not a multiple of 16 and takes the unstaged kernel."""
    rp, ci, v = cg.gen_matrix(kind, N, shift=1e-3, sigma=1.0, seed=5)
    n = len(rp) - 1
    B = cg.gen_rhs("normal", n, m, 7)
    M = cg.Matrix(rp, ci, v, want_fp32=True)
    kw = dict(s=s, bounds="gerschgorin", tol=1e-8, maxit=600, precision="mixed",
              residual="fp64")
    out = {f: _solve_dev(M, B, cg.Params(spmm_format=f, **kw))
           for f in ("auto", "dia_unstaged", "csr")}
    M.close()
    Xa, ia = out["auto"]
    for f in ("dia_unstaged", "csr"):
        X, i = out[f]
        assert i["status"] == 0 and ia["status"] == 0
        assert i["iterations"] == ia["iterations"], f
        assert np.array_equal(X, Xa), f
    assert ia["true_relres_max"] <= 1e-8


def test_dia_not_built_for_irregular_matrix(lib):
    rng = np.random.default_rng(3)
    n = 2000
    rows = [np.unique(np.concatenate([[i], rng.integers(0, n, 6)])) for i in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate(rows).astype(np.int32)
    v = rng.standard_normal(len(ci))
    M = cg.Matrix(rp, ci, v)
    assert M.diagonals() == 0
    M.close()


def test_dia_not_built_for_unsorted_rows(lib):
    rp, ci, v = cg.gen_matrix("lap2d", 20)
    ci = ci.copy()
    ci[rp[50]:rp[51]] = ci[rp[50]:rp[51]][::-1]  # one row's columns reversed
    v = v.copy()
    v[rp[50]:rp[51]] = v[rp[50]:rp[51]][::-1]
    M = cg.Matrix(rp, ci, v)
    assert M.diagonals() == 0
    M.close()


@pytest.mark.parametrize("kind,N,ndiag", [("st3d27", 96, 27), ("lap3d7", 64, 7),
                                          ("lap2d", 512, 5)])
def test_dia_view_found_on_large_grids(lib, kind, N, ndiag):
    """The offset set is exact (every nonzero hashed), independent of which
    rows are boundary rows."""
    rp, ci, v = cg.gen_matrix(kind, N)
    M = cg.Matrix(rp, ci, v)
    assert M.diagonals() == ndiag
    M.close()


@pytest.mark.parametrize("kind,N,m", [("st3d27", 24, 16), ("lap3d7", 20, 8), ("lap2d", 48, 4)])
def test_float_float_residual_replacement(lib, kind, N, m):
    """Mixed mode over a DIA view: periodic residual replacements in
    float-float reach the same tolerance as FP64 replacements, with the
    solutions within the solution tolerance and iteration counts within 2."""
    rp, ci, v = cg.gen_matrix(kind, N, shift=1e-3)
    n = len(rp) - 1
    B = cg.gen_rhs("uniform", n, m, 9, -1.0, 1.0)
    M = cg.Matrix(rp, ci, v, want_fp32=True)
    kw = dict(s=4, bounds="gerschgorin", tol=1e-10, maxit=600, precision="mixed", rr_period=3)
    Xf, inf_ = _solve_dev(M, B, cg.Params(residual="auto", **kw))
    Xd, ind = _solve_dev(M, B, cg.Params(residual="fp64", **kw))
    M.close()
    assert inf_["status"] == 0 and ind["status"] == 0
    assert inf_["true_relres_max"] <= 1e-10 and ind["true_relres_max"] <= 1e-10
    assert abs(inf_["iterations"] - ind["iterations"]) <= 2
    assert np.linalg.norm(Xf - Xd) <= 1e-7 * np.linalg.norm(Xd)
