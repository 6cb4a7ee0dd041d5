"""Tall-skinny QR (cacg_k_tsqr, CholeskyQR2 on the FP64 Gram).

The reference has no working QR (src/TSQR.c is empty, the Householder QR of
src/MatrixDecomposition.c:3-93 is unfinished and never called), so there is
no reference output to match: the checks are the factorisation's own
properties and numpy's FP64 factors of the same block.
"""
import numpy as np
import pytest

import oracle as O
from gpu_util import dev, host, ptr

pytestmark = pytest.mark.gpu


def _tsqr(lib, torch, V):
    n, k = V.shape
    dV = dev(torch, V)
    dQ = torch.zeros((n, k), dtype=torch.float64, device="cuda")
    dR = torch.zeros((k, k), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_tsqr(n, k, ptr(dV), k, ptr(dQ), k, ptr(dR), None)
    return rc, host(dQ), host(dR)


@pytest.mark.parametrize("n,k", [(20000, 8), (50000, 32), (100000, 96), (30000, 128),
                                 (4099, 13), (64, 64)])
def test_tsqr_factorises_and_orthonormalises(lib, torch_cuda, n, k):
    V = O.gen_rhs("normal", n, k, 21)
    rc, Q, R = _tsqr(lib, torch_cuda, V)
    assert rc == 0
    assert np.linalg.norm(Q @ R - V) / np.linalg.norm(V) <= 1e-13
    assert np.abs(Q.T @ Q - np.eye(k)).max() <= 1e-13 * k
    assert np.allclose(np.tril(R, -1), 0.0) and (np.diag(R) > 0).all()
    Rnp = np.linalg.cholesky(V.T @ V).T  # the same R (positive diagonal)
    assert np.linalg.norm(R - Rnp) / np.linalg.norm(Rnp) <= 1e-12


def test_tsqr_ill_conditioned_block(lib, torch_cuda):
    """cond(V) = 1e6: CholeskyQR2 stays orthogonal to working accuracy."""
    n, k = 40000, 24
    rng = np.random.default_rng(5)
    U, _ = np.linalg.qr(rng.standard_normal((n, k)))
    W, _ = np.linalg.qr(rng.standard_normal((k, k)))
    V = (U * np.logspace(0, -6, k)) @ W
    rc, Q, R = _tsqr(lib, torch_cuda, V)
    assert rc == 0
    assert np.abs(Q.T @ Q - np.eye(k)).max() <= 1e-12
    assert np.linalg.norm(Q @ R - V) / np.linalg.norm(V) <= 1e-13


def test_tsqr_rank_deficient_block_reports_breakdown(lib, torch_cuda):
    V = O.gen_rhs("normal", 5000, 8, 22)
    V[:, 5] = 0.0
    rc, _, _ = _tsqr(lib, torch_cuda, V)
    assert rc == -4  # CACG_ERR_BREAKDOWN


def test_tsqr_rejects_bad_shapes(lib, torch_cuda):
    V = np.zeros((10, 16))
    rc, _, _ = _tsqr(lib, torch_cuda, V)  # n < k
    assert rc == -1
