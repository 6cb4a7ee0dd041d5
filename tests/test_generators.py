"""Seeded generators (cacg_gb300/csrc/cacg_gen.c), shared by the GPU library
and the oracle: structure, symmetry, SPD-ness markers, determinism, and the
transcendental helpers that keep x86 and Arm hosts bit-identical."""
import math

import numpy as np
import pytest

import cacg_gb300 as cg
import oracle as O


@pytest.mark.parametrize("kind,N,nnz", [("lap2d", 128, 81408), ("lap3d7", 64, 1810432),
                                        ("st3d27", 128, 55742968),
                                        ("varcoef2d", 1024, 5238784)])
def test_nnz_formulas(kind, N, nnz):
    assert O.port_lib().cacg_gen_nnz(O.KINDS[kind], N) == nnz


@pytest.mark.parametrize("kind,N", [("lap2d", 17), ("lap3d7", 9), ("st3d27", 7),
                                    ("varcoef2d", 13)])
def test_structure_symmetric_sorted(kind, N):
    sp = pytest.importorskip("scipy.sparse")
    rp, ci, v = O.gen_matrix(kind, N, shift=1e-6, sigma=1.5, seed=3)
    n = len(rp) - 1
    for i in range(n):
        row = ci[rp[i]:rp[i + 1]]
        assert (np.diff(row) > 0).all() and i in row
    A = sp.csr_matrix((v, ci, rp), shape=(n, n))
    assert abs(A - A.T).max() == 0.0
    d = A.diagonal()
    off = np.asarray(abs(A).sum(axis=1)).ravel() - abs(d)
    assert (d - off >= -1e-12).all()  # weakly diagonally dominant -> SPD with Dirichlet rows


def test_library_and_oracle_generators_identical(lib):
    for kind in ("lap2d", "st3d27", "varcoef2d"):
        a = cg.gen_matrix(kind, 11, 1e-6, 1.5, 3)
        b = O.gen_matrix(kind, 11, 1e-6, 1.5, 3)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    assert np.array_equal(cg.gen_rhs("normal", 500, 3, 9), O.gen_rhs("normal", 500, 3, 9))


def test_rhs_distributions():
    u = O.gen_rhs("uniform", 20000, 4, 2, -1.0, 1.0)
    assert -1.0 <= u.min() and u.max() < 1.0 and abs(u.mean()) < 0.02
    z = O.gen_rhs("normal", 20000, 4, 1)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02
    b = O.gen_rhs("beta25", 20000, 4, 3)
    assert 0 < b.min() and b.max() < 1 and abs(b.mean() - 2 / 7) < 0.01
    assert np.array_equal(O.gen_rhs("normal", 100, 2, 7), O.gen_rhs("normal", 100, 2, 7))
    assert not np.array_equal(O.gen_rhs("normal", 100, 2, 7), O.gen_rhs("normal", 100, 2, 8))


def test_deterministic_log_exp():
    L = O.port_lib()
    for x in [1e-300, 1e-5, 0.3, 1.0, 2.0, 10.0, 1e10, 1e300]:
        assert abs(L.cacg_det_log(x) - math.log(x)) <= 4e-16 * max(1.0, abs(math.log(x)))
    for x in [-700.0, -5.0, -0.5, 0.0, 1e-9, 0.7, 3.0, 50.0, 700.0]:
        assert abs(L.cacg_det_exp(x) - math.exp(x)) <= 8e-16 * math.exp(x)
