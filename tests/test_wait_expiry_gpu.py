"""The expiry path of the bounded device-side waits, exercised without a
fault: the tcgen05 Gram's pipeline waits are given a poll limit of zero
(cacg_set_pipeline_wait_limit), so every one of them runs out at once.  The
kernel must drain its own TMA loads and MMAs, free its tensor memory, set
its status word and return; the entry point reports CACG_ERR_TIMEOUT, the
context stays usable, and the next call with the default limit returns the
bit-identical product.  The same through a whole mixed solve."""
import numpy as np
import pytest

import cacg_gb300 as cg
import oracle as O
from gpu_util import dev, host, ptr

pytestmark = pytest.mark.gpu

F32, TC5 = 1, 5


def _gram_tc5(lib, torch, L, R1, R2):
    n, ka = L.shape
    kb1, kb2 = R1.shape[1], R2.shape[1]
    dL, d1, d2 = dev(torch, L), dev(torch, R1), dev(torch, R2)
    Cm = torch.zeros((ka, kb1 + kb2), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, TC5, n, ptr(dL), ka, ka, ptr(d1), kb1, kb1, ptr(d2), kb2, kb2,
                         ptr(Cm), kb1 + kb2, None)
    return rc, host(Cm)


@pytest.mark.parametrize("n", [100000, 3001])
def test_gram_pipeline_wait_expiry_then_recovery(lib, torch_cuda, n):
    torch = torch_cuda
    L = O.gen_rhs("normal", n, 96, 1).astype(np.float32)
    R1 = O.gen_rhs("normal", n, 96, 2).astype(np.float32)
    R2 = O.gen_rhs("normal", n, 16, 3).astype(np.float32)
    rc0, C0 = _gram_tc5(lib, torch, L, R1, R2)
    assert rc0 == 0
    lib.cacg_set_pipeline_wait_limit(0)
    try:
        rc1, _ = _gram_tc5(lib, torch, L, R1, R2)
    finally:
        lib.cacg_set_pipeline_wait_limit(-1)
    assert rc1 == -5  # CACG_ERR_TIMEOUT
    torch.cuda.synchronize()  # the context is intact
    rc2, C2 = _gram_tc5(lib, torch, L, R1, R2)
    assert rc2 == 0
    assert np.array_equal(C0, C2)


def test_solve_reports_timeout_and_next_solve_is_unchanged(lib, torch_cuda):
    rp, ci, v = cg.gen_matrix("st3d27", 16)
    n = len(rp) - 1
    B = cg.gen_rhs("uniform", n, 16, 2, -1.0, 1.0)
    kw = dict(s=6, bounds=("given", 0.05, 52.0), tol=1e-8, maxit=300, precision="mixed")
    X0, i0 = cg.solve(rp, ci, v, B, **kw)
    lib.cacg_set_pipeline_wait_limit(0)
    try:
        with pytest.raises(cg.CacgError) as e:
            cg.solve(rp, ci, v, B, **kw)
    finally:
        lib.cacg_set_pipeline_wait_limit(-1)
    assert e.value.code == -5
    X1, i1 = cg.solve(rp, ci, v, B, **kw)
    assert i1["status"] == 0 and i1["iterations"] == i0["iterations"]
    assert np.array_equal(X0, X1)
