#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the REFERENCE solver.

Runs the reference sclc/cacg sources (compiled by oracle/build.py into
oracle/_ref/libcacgref.so, one MPI rank, -ffp-contract=off) on seeded
synthetic inputs from cacg_gb300/csrc/cacg_gen.c and stores inputs' seeds,
outputs and checksums.  The reference has no tests or fixtures of its own,
so these runs are the pin for both the CPU restatement (bit-exact) and the
GPU solver (tolerance).  Needs the reference tree; run from the repo root:

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    assert O.ref_available(), "reference sources not available"
    out = {}
    # ---- generators: structure and value checksums
    for kind, N, kw in [("lap2d", 128, {}), ("lap3d7", 64, {}), ("st3d27", 32, {}),
                        ("varcoef2d", 64, dict(shift=1e-6, sigma=1.5, seed=3))]:
        rp, ci, v = O.gen_matrix(kind, N, **kw)
        out["gen_%s_%d" % (kind, N)] = np.array(
            [sha(rp), sha(ci), sha(v)], dtype="U64")
    for dist, n, m, seed, a, b in [("uniform", 16384, 1, 0, 0.0, 1.0),
                                   ("normal", 4096, 8, 1, 0.0, 1.0),
                                   ("uniform", 4096, 16, 2, -1.0, 1.0),
                                   ("beta25", 4096, 32, 3, 0.0, 1.0)]:
        out["rhs_%s_%d_%d_%d" % (dist, n, m, seed)] = np.array(
            [sha(O.gen_rhs(dist, n, m, seed, a, b))], dtype="U64")

    # ---- config 1 in full: CBCG 2-D 5-pt 128^2, analytic bounds, tol 1e-8
    rp, ci, v = O.gen_matrix("lap2d", 128)
    B = O.gen_rhs("uniform", 16384, 1, 0)
    c = np.cos(np.pi / 129)
    bounds = (4 - 4 * c, 4 + 4 * c)
    eps = 1e-8 * np.linalg.norm(B[:, 0])
    X, it, hist, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), 4, eps, bounds, maxit=2000)
    out["cfg1_X_sha"] = np.array([sha(X)], dtype="U64")
    out["cfg1_X_rows4"] = X[::4]
    out["cfg1_iters"] = np.array([it])
    out["cfg1_hist"] = hist
    out["cfg1_relres"] = O.port_true_relres(rp, ci, v, B, X)
    out["cfg1_eps"] = np.array([eps])

    # ---- block solves at reduced grids (same families as the configurations)
    cases = {
        "b7": ("lap3d7", 24, 8, 8, "normal", 1, 0.0, 1.0, "analytic7"),
        "b27": ("st3d27", 20, 16, 6, "uniform", 2, -1.0, 1.0, (0.05, 52.0)),
        "bvc": ("varcoef2d", 32, 4, 4, "beta25", 3, 0.0, 1.0, None),
    }
    for key, (kind, N, m, s, dist, seed, a, b, bnd) in cases.items():
        kw = dict(shift=1e-6, sigma=1.5, seed=3) if kind == "varcoef2d" else {}
        rp, ci, v = O.gen_matrix(kind, N, **kw)
        n = len(rp) - 1
        B = O.gen_rhs(dist, n, m, seed, a, b)
        if bnd == "analytic7":
            c = np.cos(np.pi / (N + 1))
            bnd = (6 - 6 * c, 6 + 6 * c)
        eps = 1e-8 * np.linalg.norm(B[:, 0])
        X, it, hist, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), s, eps, bnd, maxit=400)
        out[key + "_X_sha"] = np.array([sha(X)], dtype="U64")
        out[key + "_X_rows8"] = X[::8]
        out[key + "_iters"] = np.array([it])
        out[key + "_hist"] = hist
        out[key + "_eps"] = np.array([eps])
        out[key + "_bounds"] = np.array(bnd if bnd is not None else (np.nan, np.nan))

    # ---- per-kernel vectors (small)
    rp, ci, v = O.gen_matrix("st3d27", 8)
    n = len(rp) - 1
    R = O.gen_rhs("normal", n, 4, 11)
    lo, hi = O.ref_gerschgorin(rp, ci, v)
    out["k_gersch"] = np.array([lo, hi])
    al, be = 2.0 / (hi - lo), -(hi + lo) / (hi - lo)
    out["k_basis"] = O.ref_basis(rp, ci, v, R, 5, al, be)
    out["k_spmm"] = O.ref_spmm(rp, ci, v, O.gen_rhs("normal", n, 12, 12))
    L = O.gen_rhs("normal", 300, 20, 13)
    Rm = O.gen_rhs("normal", 300, 24, 14)
    out["k_gram"] = O.ref_gram(L, Rm)
    W = O.gen_rhs("normal", 20, 24, 15)
    out["k_tallsmall"] = O.ref_tallsmall(L, W)
    G = O.gen_rhs("normal", 80, 20, 16)
    Mx = G.T @ G / 80 + np.eye(20)
    out["k_lu_M"] = Mx
    out["k_lu"] = O.ref_lu(Mx, O.gen_rhs("normal", 20, 6, 17))
    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_golden.npz"),
          "cfg1 its", int(out["cfg1_iters"][0]),
          {k: int(out[k + "_iters"][0]) for k in cases})


if __name__ == "__main__":
    main()
