"""The oracle is pinned before it is trusted.

* The project's C restatement (oracle/cacg_oracle.c) reproduces the reference
  solver (sclc/cacg src/*.c compiled as shipped by oracle/build.py) BIT FOR BIT
  on one rank, kernel by kernel and for whole CBCG/BCBCG solves.
* Both reproduce the committed fixtures tests/golden/reference_golden.npz
  (made by tests/golden/make_golden.py from the reference): generator
  checksums, the full config-1 solve, three reduced block solves, kernels.
"""
import hashlib
import os

import numpy as np
import pytest

import oracle as O

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz"))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference sources not staged")


def test_generator_checksums():
    for kind, N, kw in [("lap2d", 128, {}), ("lap3d7", 64, {}), ("st3d27", 32, {}),
                        ("varcoef2d", 64, dict(shift=1e-6, sigma=1.5, seed=3))]:
        rp, ci, v = O.gen_matrix(kind, N, **kw)
        assert list(G["gen_%s_%d" % (kind, N)]) == [sha(rp), sha(ci), sha(v)], kind
    for dist, n, m, seed, a, b in [("uniform", 16384, 1, 0, 0.0, 1.0),
                                   ("normal", 4096, 8, 1, 0.0, 1.0),
                                   ("uniform", 4096, 16, 2, -1.0, 1.0),
                                   ("beta25", 4096, 32, 3, 0.0, 1.0)]:
        assert G["rhs_%s_%d_%d_%d" % (dist, n, m, seed)][0] == sha(
            O.gen_rhs(dist, n, m, seed, a, b))


def test_port_config1_matches_golden():
    rp, ci, v = O.gen_matrix("lap2d", 128)
    B = O.gen_rhs("uniform", 16384, 1, 0)
    c = np.cos(np.pi / 129)
    eps = float(G["cfg1_eps"][0])
    assert eps == 1e-8 * np.linalg.norm(B[:, 0])
    X, it, hist = O.port_solve(rp, ci, v, B, np.zeros_like(B), 4, eps,
                               (4 - 4 * c, 4 + 4 * c), maxit=2000)
    assert it == int(G["cfg1_iters"][0]) == 96
    assert sha(X) == G["cfg1_X_sha"][0]
    assert np.array_equal(hist, G["cfg1_hist"])
    assert np.array_equal(X[::4], G["cfg1_X_rows4"])
    assert G["cfg1_relres"][0] < 1e-8


@pytest.mark.parametrize("key,kind,N,m,s,dist,seed,a,b", [
    ("b7", "lap3d7", 24, 8, 8, "normal", 1, 0.0, 1.0),
    ("b27", "st3d27", 20, 16, 6, "uniform", 2, -1.0, 1.0),
    ("bvc", "varcoef2d", 32, 4, 4, "beta25", 3, 0.0, 1.0)])
def test_port_block_solves_match_golden(key, kind, N, m, s, dist, seed, a, b):
    kw = dict(shift=1e-6, sigma=1.5, seed=3) if kind == "varcoef2d" else {}
    rp, ci, v = O.gen_matrix(kind, N, **kw)
    n = len(rp) - 1
    B = O.gen_rhs(dist, n, m, seed, a, b)
    bnd = G[key + "_bounds"]
    bounds = None if np.isnan(bnd[0]) else (float(bnd[0]), float(bnd[1]))
    X, it, hist = O.port_solve(rp, ci, v, B, np.zeros_like(B), s, float(G[key + "_eps"][0]),
                               bounds, maxit=400)
    assert it == int(G[key + "_iters"][0])
    assert sha(X) == G[key + "_X_sha"][0]
    assert np.array_equal(hist, G[key + "_hist"])


def test_port_kernels_match_golden():
    rp, ci, v = O.gen_matrix("st3d27", 8)
    n = len(rp) - 1
    R = O.gen_rhs("normal", n, 4, 11)
    lo, hi = O.port_gerschgorin(rp, ci, v)
    assert np.array_equal([lo, hi], G["k_gersch"])
    al, be = 2.0 / (hi - lo), -(hi + lo) / (hi - lo)
    assert np.array_equal(O.port_basis(rp, ci, v, R, 5, al, be), G["k_basis"])
    assert np.array_equal(O.port_spmm(rp, ci, v, O.gen_rhs("normal", n, 12, 12)), G["k_spmm"])
    L = O.gen_rhs("normal", 300, 20, 13)
    assert np.array_equal(O.port_gram(L, O.gen_rhs("normal", 300, 24, 14)), G["k_gram"])
    assert np.array_equal(O.port_tallsmall(L, O.gen_rhs("normal", 20, 24, 15)),
                          G["k_tallsmall"])
    assert np.array_equal(O.port_lu(G["k_lu_M"], O.gen_rhs("normal", 20, 6, 17)), G["k_lu"])


@needs_ref
@pytest.mark.parametrize("kind,N,m,s,bounds", [("lap2d", 40, 1, 4, None),
                                               ("lap2d", 40, 1, 6, (0.01, 8.0)),
                                               ("lap3d7", 12, 8, 8, None),
                                               ("st3d27", 10, 16, 6, (0.05, 52.0)),
                                               ("lap3d7", 10, 3, 5, None)])
def test_port_equals_reference_bitwise(kind, N, m, s, bounds):
    rp, ci, v = O.gen_matrix(kind, N)
    n = len(rp) - 1
    B = O.gen_rhs("normal", n, m, 5)
    eps = 1e-9 * np.linalg.norm(B[:, 0])
    Xr, itr, hr, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), s, eps, bounds, maxit=300)
    Xp, itp, hp = O.port_solve(rp, ci, v, B, np.zeros_like(B), s, eps, bounds, maxit=300)
    assert itr == itp
    assert np.array_equal(Xr, Xp)
    assert np.array_equal(hr, hp)


@needs_ref
def test_port_kernels_equal_reference_bitwise():
    rp, ci, v = O.gen_matrix("varcoef2d", 20, shift=1e-6, sigma=1.5, seed=3)
    n = len(rp) - 1
    assert np.array_equal(O.port_gerschgorin(rp, ci, v), O.ref_gerschgorin(rp, ci, v))
    X = O.gen_rhs("normal", n, 7, 1)
    assert np.array_equal(O.port_spmm(rp, ci, v, X), O.ref_spmm(rp, ci, v, X))
    for m, s, cb in [(1, 4, True), (7, 3, False), (2, 6, False)]:
        R = O.gen_rhs("normal", n, m, 2)
        assert np.array_equal(O.port_basis(rp, ci, v, R, s, 0.3, -1.1),
                              O.ref_basis(rp, ci, v, R, s, 0.3, -1.1, cbcg=cb))
    L, Rm = O.gen_rhs("normal", 500, 9, 3), O.gen_rhs("normal", 500, 11, 4)
    assert np.array_equal(O.port_gram(L, Rm), O.ref_gram(L, Rm))
    Sq = O.gen_rhs("normal", 500, 9, 5)
    assert np.array_equal(O.ref_gram(L, Sq, square=True), O.port_gram(L, Sq))
    W = O.gen_rhs("normal", 9, 4, 6)
    assert np.array_equal(O.port_tallsmall(L, W), O.ref_tallsmall(L, W))
    M = L.T @ L / 500 + np.eye(9)
    assert np.array_equal(O.port_lu(M, W), O.ref_lu(M, W))


@needs_ref
def test_reference_reproduces_golden():
    rp, ci, v = O.gen_matrix("lap2d", 128)
    B = O.gen_rhs("uniform", 16384, 1, 0)
    c = np.cos(np.pi / 129)
    X, it, hist, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), 4, float(G["cfg1_eps"][0]),
                                 (4 - 4 * c, 4 + 4 * c), maxit=2000)
    assert it == 96 and sha(X) == G["cfg1_X_sha"][0]


@needs_ref
def test_reference_multirank_shim_agrees():
    """The threaded MPI shim runs the reference on several ranks (block-row
    distribution of src/SparseMatrixDistribution.c:64-87): same answer to
    rounding, the reduction order being the only difference."""
    rp, ci, v = O.gen_matrix("lap3d7", 14)
    n = len(rp) - 1
    B = O.gen_rhs("normal", n, 4, 1)
    eps = 1e-8 * np.linalg.norm(B[:, 0])
    X1, it1, _, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), 4, eps, None, 200, nranks=1)
    X3, it3, _, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), 4, eps, None, 200, nranks=3)
    assert abs(it1 - it3) <= 1
    assert np.linalg.norm(X1 - X3) / np.linalg.norm(X1) < 1e-9


def test_breakdown_injected_in_oracle_is_silent_nan():
    """A planted fault (zero RHS column -> singular Q^T A Q) makes the
    reference algorithm produce NaN silently; the GPU library reports
    CACG_ERR_BREAKDOWN for the same input (tests/test_solver_gpu.py)."""
    rp, ci, v = O.gen_matrix("lap2d", 12)
    B = O.gen_rhs("normal", 144, 3, 1)
    B[:, 1] = 0.0
    X, it, hist = O.port_solve(rp, ci, v, B, np.zeros_like(B), 4, 1e-10, None, maxit=5)
    assert not np.isfinite(X).all()
