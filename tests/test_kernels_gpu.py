"""Kernel-level parity: each libcacg.so kernel (called through its C ABI entry
point) against the oracle's restatement of the reference routine on the same
seeded inputs.

Tolerances (FP64 kernels differ from the reference only in summation order and
fused multiply-add): normwise relative error <= 1e-12.  FP32 kernels are
compared with the FP64 evaluation of the same FP32 inputs: <= 2e-6.
"""
import numpy as np
import pytest

import oracle as O
from gpu_util import dev, host, ptr, relerr

pytestmark = pytest.mark.gpu

F64, F32 = 0, 1


def _mat(kind="st3d27", N=10, **kw):
    return O.gen_matrix(kind, N, **kw)


@pytest.mark.parametrize("kind,N", [("lap2d", 40), ("lap3d7", 12), ("st3d27", 10),
                                    ("varcoef2d", 30)])
@pytest.mark.parametrize("w", [1, 2, 3, 8, 16, 24, 32, 96, 130])
def test_spmm_f64_matches_reference(lib, torch_cuda, kind, N, w):
    torch = torch_cuda
    rp, ci, v = _mat(kind, N, shift=1e-6, sigma=1.5, seed=3)
    n = len(rp) - 1
    X = O.gen_rhs("normal", n, w, 7)
    Z1 = O.gen_rhs("normal", n, w, 8)
    Z2 = O.gen_rhs("normal", n, w, 9)
    want_plain = O.ref_spmm(rp, ci, v, X) if O.ref_available() else O.port_spmm(rp, ci, v, X)
    ca, cb, cc = 0.7, -1.3, -1.0
    want = ca * want_plain + cb * Z1 + cc * Z2
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci, v=v, X=X, Z1=Z1, Z2=Z2).items()}
    Y = torch.empty((n, w), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_spmm(F64, n, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), w, ptr(d["X"]), w,
                         ptr(Y), w, ptr(d["Z1"]), w, ptr(d["Z2"]), w, ca, cb, cc, None)
    assert rc == 0
    assert relerr(host(Y), want) <= 1e-13
    Y0 = torch.empty((n, w), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_spmm(F64, n, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), w, ptr(d["X"]), w,
                         ptr(Y0), w, None, 0, None, 0, 1.0, 0.0, 0.0, None)
    assert rc == 0
    assert relerr(host(Y0), want_plain) <= 1e-13


@pytest.mark.parametrize("w", [1, 4, 5, 16, 32, 96])
def test_spmm_f32(lib, torch_cuda, w):
    torch = torch_cuda
    rp, ci, v = _mat("st3d27", 12)
    n = len(rp) - 1
    X = O.gen_rhs("uniform", n, w, 3, -1.0, 1.0).astype(np.float32)
    v32 = v.astype(np.float32)
    want = O.port_spmm(rp, ci, v32.astype(np.float64), X.astype(np.float64))
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci, v=v32, X=X).items()}
    Y = torch.empty((n, w), dtype=torch.float32, device="cuda")
    rc = lib.cacg_k_spmm(F32, n, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), w, ptr(d["X"]), w,
                         ptr(Y), w, None, 0, None, 0, 1.0, 0.0, 0.0, None)
    assert rc == 0
    assert relerr(host(Y), want) <= 2e-6


def _irregular_csr(n, seed):
    """Random CSR with empty rows, short rows and a few rows of ~600 entries
    (a warp block of such rows exceeds the staged-entry capacity)."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, n)
    lens[rng.choice(n, 5, replace=False)] = 600
    lens[rng.choice(n, 7, replace=False)] = 0
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate([np.sort(rng.choice(n, int(L), replace=False)) for L in lens]).astype(np.int32)
    v = rng.standard_normal(int(rp[-1]))
    return rp, ci, v


@pytest.mark.parametrize("w", [2, 16, 96])
@pytest.mark.parametrize("f32", [False, True])
def test_spmm_irregular_rows(lib, torch_cuda, w, f32):
    torch = torch_cuda
    n = 5003
    rp, ci, v = _irregular_csr(n, 21)
    dt = np.float32 if f32 else np.float64
    X = O.gen_rhs("normal", n, w, 22).astype(dt)
    Z1 = O.gen_rhs("normal", n, w, 23).astype(dt)
    vv = v.astype(dt)
    want = 0.5 * O.port_spmm(rp, ci, vv.astype(np.float64), X.astype(np.float64)) \
        - 2.0 * Z1.astype(np.float64)
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci, v=vv, X=X, Z1=Z1).items()}
    Y = torch.empty((n, w), dtype=torch.float32 if f32 else torch.float64, device="cuda")
    rc = lib.cacg_k_spmm(F32 if f32 else F64, n, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), w,
                         ptr(d["X"]), w, ptr(Y), w, ptr(d["Z1"]), w, None, 0, 0.5, -2.0, 0.0, None)
    assert rc == 0
    assert relerr(host(Y), want) <= (5e-6 if f32 else 1e-13)


@pytest.mark.parametrize("w", [3, 16])
def test_spmm_unaligned_index_arrays(lib, torch_cuda, w):
    """ci / val starting off a 16-byte boundary take the unstaged path."""
    torch = torch_cuda
    rp, ci, v = _mat("st3d27", 9)
    n = len(rp) - 1
    X = O.gen_rhs("normal", n, w, 24)
    want = O.port_spmm(rp, ci, v, X)
    ci_pad = np.concatenate([np.zeros(1, np.int32), ci])
    v_pad = np.concatenate([np.zeros(1), v])
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci_pad, v=v_pad, X=X).items()}
    Y = torch.empty((n, w), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_spmm(F64, n, ptr(d["rp"]), ptr(d["ci"]) + 4, ptr(d["v"]) + 8, w, ptr(d["X"]),
                         w, ptr(Y), w, None, 0, None, 0, 1.0, 0.0, 0.0, None)
    assert rc == 0
    assert relerr(host(Y), want) <= 1e-13


@pytest.mark.parametrize("kind,N,m,s", [("lap2d", 48, 1, 4), ("lap3d7", 12, 8, 8),
                                        ("st3d27", 10, 16, 6), ("lap3d7", 10, 3, 5)])
def test_basis_matches_reference(lib, torch_cuda, kind, N, m, s):
    torch = torch_cuda
    rp, ci, v = _mat(kind, N)
    n = len(rp) - 1
    R = O.gen_rhs("normal", n, m, 11)
    lo, hi = O.port_gerschgorin(rp, ci, v)
    alpha, beta = 2.0 / (hi - lo), -(hi + lo) / (hi - lo)
    if O.ref_available():
        want = O.ref_basis(rp, ci, v, R, s, alpha, beta, cbcg=(m == 1))
    else:
        want = O.port_basis(rp, ci, v, R, s, alpha, beta)
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci, v=v, R=R).items()}
    S = torch.zeros((n, s * m), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_basis(F64, n, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), ptr(d["R"]), m, s,
                          alpha, beta, ptr(S), s * m, None)
    assert rc == 0
    assert relerr(host(S), want) <= 1e-12


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("n,ka,kb1,kb2", [(20000, 64, 64, 8), (50000, 96, 96, 16),
                                          (3001, 12, 12, 3), (40000, 128, 128, 32),
                                          (7, 4, 4, 1)])
def test_gram_f64_matches_reference(lib, torch_cuda, variant, n, ka, kb1, kb2):
    torch = torch_cuda
    L = O.gen_rhs("normal", n, ka, 1)
    R1 = O.gen_rhs("normal", n, kb1, 2)
    R2 = O.gen_rhs("normal", n, kb2, 3)
    want = O.port_gram(L, np.hstack([R1, R2]))
    if O.ref_available() and n * ka <= 2_000_000:
        assert np.array_equal(want, O.ref_gram(L, np.hstack([R1, R2])))
    d = {k: dev(torch, a) for k, a in dict(L=L, R1=R1, R2=R2).items()}
    C = torch.zeros((ka, kb1 + kb2), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F64, variant, n, ptr(d["L"]), ka, ka, ptr(d["R1"]), kb1, kb1,
                         ptr(d["R2"]), kb2, kb2, ptr(C), kb1 + kb2, None)
    assert rc == 0
    assert relerr(host(C), want) <= 1e-12


@pytest.mark.parametrize("n,ka,kb1,kb2", [(100000, 96, 96, 16), (5000, 24, 24, 4)])
def test_gram_f32_fp64_accumulation(lib, torch_cuda, n, ka, kb1, kb2):
    """FP32 inputs, FP64-accurate accumulation: matches the exact (FP64) Gram
    of the FP32 values far below FP32 rounding."""
    torch = torch_cuda
    L = O.gen_rhs("normal", n, ka, 4).astype(np.float32)
    R1 = O.gen_rhs("normal", n, kb1, 5).astype(np.float32)
    R2 = O.gen_rhs("normal", n, kb2, 6).astype(np.float32)
    want = O.port_gram(L.astype(np.float64), np.hstack([R1, R2]).astype(np.float64))
    d = {k: dev(torch, a) for k, a in dict(L=L, R1=R1, R2=R2).items()}
    C = torch.zeros((ka, kb1 + kb2), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, 0, n, ptr(d["L"]), ka, ka, ptr(d["R1"]), kb1, kb1, ptr(d["R2"]),
                         kb2, kb2, ptr(C), kb1 + kb2, None)
    assert rc == 0
    assert relerr(host(C), want) <= 1e-10


@pytest.mark.parametrize("vt", [F64, F32])
@pytest.mark.parametrize("n,k", [(10000, 64), (30000, 96), (999, 12), (5000, 256)])
def test_qupdate(lib, torch_cuda, vt, n, k):
    torch = torch_cuda
    Q = O.gen_rhs("normal", n, k, 1)
    S = O.gen_rhs("normal", n, k, 2)
    beta = O.gen_rhs("normal", k, k, 3)
    dt = np.float64 if vt == F64 else np.float32
    Qh, Sh = Q.astype(dt), S.astype(dt)
    bh = beta if vt == F64 else beta.astype(np.float32).astype(np.float64)
    want = Sh.astype(np.float64) - O.port_tallsmall(Qh.astype(np.float64), bh)
    if vt == F64 and O.ref_available():
        assert relerr(O.ref_tallsmall(Q, beta), O.port_tallsmall(Q, beta)) == 0.0
    dq, ds, db = dev(torch, Qh), dev(torch, Sh), dev(torch, beta)
    rc = lib.cacg_k_qupdate(vt, n, k, ptr(dq), k, ptr(ds), k, ptr(db), None)
    assert rc == 0
    assert relerr(host(dq), want) <= (1e-13 if vt == F64 else 3e-6)


TC5 = 32


@pytest.mark.parametrize("n,k", [(10000, 64), (30000, 96), (999, 16), (4099, 48), (127, 32),
                                 (200001, 96)])
def test_qupdate_tcgen05(lib, torch_cuda, n, k):
    """Q = S - Q beta on the tcgen05 tensor cores (bf16x3 slices, six products,
    FP32 accumulation): within 3e-6 of the FP64 product of the FP32 inputs,
    like the CUDA-core FP32 kernel."""
    torch = torch_cuda
    Qh = O.gen_rhs("normal", n, k, 1).astype(np.float32)
    Sh = O.gen_rhs("normal", n, k, 2).astype(np.float32)
    beta = O.gen_rhs("normal", k, k, 3)
    bh = beta.astype(np.float32).astype(np.float64)
    want = Sh.astype(np.float64) - O.port_tallsmall(Qh.astype(np.float64), bh)
    dq, ds, db = dev(torch, Qh), dev(torch, Sh), dev(torch, beta)
    rc = lib.cacg_k_qupdate(F32 | TC5, n, k, ptr(dq), k, ptr(ds), k, ptr(db), None)
    assert rc == 0
    assert relerr(host(dq), want) <= 3e-6


CPASYNC = 64


@pytest.mark.parametrize("n,k", [(30000, 96), (999, 16), (4099, 48), (127, 32), (200001, 96),
                                 (129, 80), (70000, 64)])
def test_qupdate_tcgen05_tma_matches_cp_async(lib, torch_cuda, n, k):
    """The TMA-fed, warp-specialised Q update and the cp.async-fed kernel
    issue the same MMAs in the same order: bit-identical outputs (row
    counts not a multiple of the 128-row tile, k not a multiple of 32)."""
    torch = torch_cuda
    Qh = O.gen_rhs("normal", n, k, 11).astype(np.float32)
    Sh = O.gen_rhs("normal", n, k, 12).astype(np.float32)
    beta = O.gen_rhs("normal", k, k, 13)
    out = []
    for vt in (F32 | TC5, F32 | TC5 | CPASYNC):
        dq, ds, db = dev(torch, Qh), dev(torch, Sh), dev(torch, beta)
        assert lib.cacg_k_qupdate(vt, n, k, ptr(dq), k, ptr(ds), k, ptr(db), None) == 0
        out.append(host(dq))
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("k", [12, 112, 128])
def test_qupdate_tcgen05_rejects_unsupported_widths(lib, torch_cuda, k):
    torch = torch_cuda
    n = 100
    dq = torch.zeros((n, k), dtype=torch.float32, device="cuda")
    ds = torch.zeros((n, k), dtype=torch.float32, device="cuda")
    db = torch.zeros((k, k), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_qupdate(F32 | TC5, n, k, ptr(dq), k, ptr(ds), k, ptr(db), None)
    assert rc == -6


@pytest.mark.parametrize("vt,exact", [(F64, False), (F64, True), (F32, False), (F32, True)])
@pytest.mark.parametrize("n,k,m", [(10000, 64, 8), (20000, 96, 16), (777, 4, 1),
                                   (3000, 15, 5), (4000, 256, 32)])
def test_xrupdate(lib, torch_cuda, vt, exact, n, k, m):
    """FP64: FP64 products.  FP32 inputs: float-float sums (exact=True) are
    FP64-accurate; the default FP32-FMA sums carry FP32 rounding of the
    k-term products only (X and R themselves are updated in FP64)."""
    torch = torch_cuda
    dt = np.float64 if vt == F64 else np.float32
    Q = O.gen_rhs("normal", n, k, 1).astype(dt)
    AQ = O.gen_rhs("normal", n, k, 2).astype(dt)
    al = O.gen_rhs("normal", k, m, 3)
    X = O.gen_rhs("normal", n, m, 4)
    R = O.gen_rhs("normal", n, m, 5)
    Xw = X + O.port_tallsmall(Q.astype(np.float64), al)
    Rw = R - O.port_tallsmall(AQ.astype(np.float64), al)
    dQ, dAQ, dal, dX, dR = (dev(torch, a) for a in (Q, AQ, al, X, R))
    S0 = torch.zeros((n, k), dtype=torch.float64 if vt == F64 else torch.float32, device="cuda")
    norms = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_xrupdate(vt | (16 if exact else 0), n, k, m, ptr(dQ), ptr(dAQ), k,
                             ptr(dal), ptr(dX), ptr(dR), ptr(S0), k, ptr(norms), None)
    assert rc == 0
    tol = 1e-13 if vt == F64 else (1e-11 if exact else 5e-6)
    assert relerr(host(dX), Xw) <= tol
    assert relerr(host(dR), Rw) <= tol
    Rg = host(dR)
    assert relerr(host(S0)[:, :m], Rg) <= (0 if vt == F64 else 1e-7)
    assert relerr(host(norms), (Rg * Rg).sum(axis=0)) <= 1e-13


@pytest.mark.parametrize("n,k", [(130001, 96), (999, 48), (5000, 100), (3001, 128), (64, 16),
                                 (20000, 96)])
def test_xrupdate_m16_tma(lib, torch_cuda, n, k):
    """FP32, 16 right-hand sides: the TMA-fed X/R update (64-row tiles, rows
    not a multiple of the tile, k not a multiple of the 32-column box) within
    the FP32-product tolerance; S0 = (float)R; norms of the new R in FP64."""
    torch = torch_cuda
    m = 16
    Q = O.gen_rhs("normal", n, k, 21).astype(np.float32)
    AQ = O.gen_rhs("normal", n, k, 22).astype(np.float32)
    al = O.gen_rhs("normal", k, m, 23)
    X = O.gen_rhs("normal", n, m, 24)
    R = O.gen_rhs("normal", n, m, 25)
    Xw = X + O.port_tallsmall(Q.astype(np.float64), al)
    Rw = R - O.port_tallsmall(AQ.astype(np.float64), al)
    dQ, dAQ, dal, dX, dR = (dev(torch, a) for a in (Q, AQ, al, X, R))
    S0 = torch.zeros((n, k), dtype=torch.float32, device="cuda")
    norms = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_xrupdate(F32, n, k, m, ptr(dQ), ptr(dAQ), k, ptr(dal), ptr(dX), ptr(dR),
                             ptr(S0), k, ptr(norms), None)
    assert rc == 0
    assert relerr(host(dX), Xw) <= 5e-6
    assert relerr(host(dR), Rw) <= 5e-6
    Rg = host(dR)
    assert relerr(host(S0)[:, :m], Rg) <= 1e-7
    assert np.all(host(S0)[:, m:] == 0)
    assert relerr(host(norms), (Rg * Rg).sum(axis=0)) <= 1e-13


FFSTATE = 128


@pytest.mark.parametrize("n,k", [(130001, 96), (999, 48), (300000, 96)])
def test_xrupdate_ffstate_matches_fp64(lib, torch_cuda, n, k):
    """X and R as float-float pairs (the mixed solve's state): the same update
    as the FP64-state kernel to the pairs' precision (about 2^-48), the same
    S0 and norms to FP32 rounding, and bit-identical on repeated calls."""
    torch = torch_cuda
    m = 16
    Q = O.gen_rhs("normal", n, k, 31).astype(np.float32)
    AQ = O.gen_rhs("normal", n, k, 32).astype(np.float32)
    al = O.gen_rhs("normal", k, m, 33)
    X0 = O.gen_rhs("normal", n, m, 34)
    R0 = O.gen_rhs("normal", n, m, 35)
    dQ, dAQ, dal = dev(torch, Q), dev(torch, AQ), dev(torch, al)

    # FP64 state
    dX, dR = dev(torch, X0), dev(torch, R0)
    S0a = torch.zeros((n, k), dtype=torch.float32, device="cuda")
    na = torch.zeros(m, dtype=torch.float64, device="cuda")
    assert lib.cacg_k_xrupdate(F32, n, k, m, ptr(dQ), ptr(dAQ), k, ptr(dal), ptr(dX), ptr(dR),
                               ptr(S0a), k, ptr(na), None) == 0
    X1, R1 = host(dX), host(dR)

    def pair(x):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
        return np.concatenate([hi.ravel(), lo.ravel()])

    def join(p):
        return p[:n * m].astype(np.float64).reshape(n, m) + p[n * m:].astype(np.float64).reshape(n, m)

    outs = []
    for _ in range(3):
        px, pr = dev(torch, pair(X0)), dev(torch, pair(R0))
        S0b = torch.zeros((n, k), dtype=torch.float32, device="cuda")
        nb = torch.zeros(m, dtype=torch.float64, device="cuda")
        assert lib.cacg_k_xrupdate(F32 | FFSTATE, n, k, m, ptr(dQ), ptr(dAQ), k, ptr(dal),
                                   ptr(px), ptr(pr), ptr(S0b), k, ptr(nb), None) == 0
        outs.append((host(px), host(pr), host(S0b), host(nb)))
    for o in outs[1:]:
        assert all(np.array_equal(a, b) for a, b in zip(outs[0], o))
    px, pr, S0b, nb = outs[0]
    assert relerr(join(px), X1) <= 1e-13
    assert relerr(join(pr), R1) <= 1e-13
    assert np.max(np.abs(S0b[:, :m] - host(S0a)[:, :m])) <= 2e-7 * np.max(np.abs(R1))
    assert relerr(nb, host(na)) <= 1e-12


@pytest.mark.parametrize("n,k,m", [(10000, 64, 8), (20000, 96, 16), (777, 4, 1),
                                   (3000, 20, 4), (4000, 256, 16), (130001, 96, 16),
                                   (5001, 32, 2)])
def test_xrupdate_tcgen05(lib, torch_cuda, n, k, m):
    """X += Q alpha, R -= AQ alpha with the products on the tcgen05 tensor
    cores (bf16x3 slices, FP32 accumulation; X, R updated in FP64): within
    the FP32-product tolerance of the CUDA-core kernel; S0 = (float)R; norms
    of the new R in FP64."""
    torch = torch_cuda
    Q = O.gen_rhs("normal", n, k, 1).astype(np.float32)
    AQ = O.gen_rhs("normal", n, k, 2).astype(np.float32)
    al = O.gen_rhs("normal", k, m, 3)
    X = O.gen_rhs("normal", n, m, 4)
    R = O.gen_rhs("normal", n, m, 5)
    Xw = X + O.port_tallsmall(Q.astype(np.float64), al)
    Rw = R - O.port_tallsmall(AQ.astype(np.float64), al)
    dQ, dAQ, dal, dX, dR = (dev(torch, a) for a in (Q, AQ, al, X, R))
    S0 = torch.zeros((n, k), dtype=torch.float32, device="cuda")
    norms = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_xrupdate(F32 | TC5, n, k, m, ptr(dQ), ptr(dAQ), k, ptr(dal), ptr(dX),
                             ptr(dR), ptr(S0), k, ptr(norms), None)
    assert rc == 0
    assert relerr(host(dX), Xw) <= 5e-6
    assert relerr(host(dR), Rw) <= 5e-6
    Rg = host(dR)
    assert relerr(host(S0)[:, :m], Rg) <= 1e-7
    assert relerr(host(norms), (Rg * Rg).sum(axis=0)) <= 1e-13


@pytest.mark.parametrize("m", [32, 5])
def test_xrupdate_tcgen05_rejects_unsupported_widths(lib, torch_cuda, m):
    torch = torch_cuda
    n, k = 100, 64
    z = lambda *sh, dt=torch.float32: torch.zeros(sh, dtype=dt, device="cuda")
    rc = lib.cacg_k_xrupdate(F32 | TC5, n, k, m, ptr(z(n, k)), ptr(z(n, k)), k,
                             ptr(z(k, m, dt=torch.float64)), ptr(z(n, m, dt=torch.float64)),
                             ptr(z(n, m, dt=torch.float64)), ptr(z(n, k)), k,
                             ptr(z(m, dt=torch.float64)), None)
    assert rc == -6


@pytest.mark.parametrize("k,r", [(4, 1), (64, 64), (64, 8), (96, 96), (96, 16), (128, 32),
                                 (200, 20), (256, 32)])
def test_lu_matches_reference(lib, torch_cuda, k, r):
    torch = torch_cuda
    G = O.gen_rhs("normal", 4 * k, k, 1)
    M = G.T @ G / (4 * k) + np.eye(k)  # SPD, like Q^T A Q
    RHS = O.gen_rhs("normal", k, r, 2)
    want = O.ref_lu(M, RHS) if O.ref_available() else O.port_lu(M, RHS)
    assert np.array_equal(want, O.port_lu(M, RHS))
    dM, dR = dev(torch, M), dev(torch, RHS)
    Y = torch.zeros((k, r), dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.cacg_k_lu(k, ptr(dM), r, ptr(dR), ptr(Y), ptr(st), None)
    assert rc == 0
    assert int(host(st)[0]) == 0
    assert relerr(host(Y), want) <= 1e-11


def test_lu_zero_pivot_sets_status(lib, torch_cuda):
    torch = torch_cuda
    k = 8
    M = np.eye(k)
    M[3, 3] = 0.0  # zero pivot: the reference divides by zero silently
    dM, dR = dev(torch, M), dev(torch, np.ones((k, 2)))
    Y = torch.zeros((k, 2), dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.cacg_k_lu(k, ptr(dM), 2, ptr(dR), ptr(Y), ptr(st), None)
    assert rc == 0
    assert int(host(st)[0]) & 1


@pytest.mark.parametrize("kind,N", [("lap2d", 64), ("st3d27", 12), ("varcoef2d", 40)])
def test_gerschgorin_exact(lib, torch_cuda, kind, N):
    torch = torch_cuda
    rp, ci, v = _mat(kind, N, shift=1e-6, sigma=1.5, seed=3)
    want = O.ref_gerschgorin(rp, ci, v) if O.ref_available() else O.port_gerschgorin(rp, ci, v)
    d = {k: dev(torch, a) for k, a in dict(rp=rp, ci=ci, v=v).items()}
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gerschgorin(len(rp) - 1, ptr(d["rp"]), ptr(d["ci"]), ptr(d["v"]), ptr(out),
                                None)
    assert rc == 0
    got = host(out)
    # min/max of per-row sums: per-row sums are formed in the reference order
    assert np.allclose(got, want, rtol=1e-14, atol=0)


@pytest.mark.parametrize("variant", [3, 4, 5])
@pytest.mark.parametrize("n,ka,kb1,kb2", [(100000, 96, 96, 16), (200000, 96, 96, 0),
                                          (5000, 24, 24, 4), (40000, 64, 64, 8),
                                          (30000, 128, 128, 32), (3001, 12, 12, 3), (33, 4, 4, 1),
                                          (20000, 160, 160, 16)])
def test_gram_tensor_core_bf16_slices(lib, torch_cuda, variant, n, ka, kb1, kb2):
    """FP32 inputs on the bf16 tensor cores (three slices, six products,
    FP32 over 256-row (mma.sync) or 64-row (tcgen05) groups, FP64 across):
    normwise within 4e-6 of the exact FP64 Gram of the FP32 values (FP32
    accumulation inside the tensor core)."""
    torch = torch_cuda
    if variant == 4 and (ka % 8 or kb1 % 8 or kb2 % 8):
        pytest.skip("slice planes need widths that are multiples of 8")
    L = O.gen_rhs("normal", n, ka, 4).astype(np.float32)
    R1 = O.gen_rhs("normal", n, kb1, 5).astype(np.float32)
    R2 = O.gen_rhs("normal", n, max(kb2, 1), 6).astype(np.float32)[:, :kb2]
    want = O.port_gram(L.astype(np.float64), np.hstack([R1, R2]).astype(np.float64))
    d = {k_: dev(torch, a) for k_, a in dict(L=L, R1=R1, R2=R2).items()}
    C = torch.zeros((ka, kb1 + kb2), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, variant, n, ptr(d["L"]), ka, ka, ptr(d["R1"]), kb1, kb1,
                         ptr(d["R2"]) if kb2 else None, kb2 if kb2 else 8, kb2, ptr(C), kb1 + kb2,
                         None)
    assert rc == 0
    assert relerr(host(C), want) <= 4e-6


@pytest.mark.parametrize("n", [7, 4099, 70001])
def test_gram_tc5_padded_rows_partial_chunks(lib, torch_cuda, n):
    """tcgen05 Gram on sub-blocks of wider arrays: L = 6 of 8 columns,
    R1 = 4 of 8, R2 = 3 of 4 (16-byte row copies that end inside a chunk are
    zero-filled past the block's last column)."""
    torch = torch_cuda
    Lw = O.gen_rhs("normal", n, 8, 11).astype(np.float32)
    R1w = O.gen_rhs("normal", n, 8, 12).astype(np.float32)
    R2w = O.gen_rhs("normal", n, 4, 13).astype(np.float32)
    want = O.port_gram(Lw[:, :6].astype(np.float64),
                       np.hstack([R1w[:, :4], R2w[:, :3]]).astype(np.float64))
    d = {k_: dev(torch, a) for k_, a in dict(L=Lw, R1=R1w, R2=R2w).items()}
    C = torch.zeros((6, 7), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, 5, n, ptr(d["L"]), 8, 6, ptr(d["R1"]), 8, 4, ptr(d["R2"]), 4, 3,
                         ptr(C), 7, None)
    assert rc == 0
    assert relerr(host(C), want) <= 4e-6


@pytest.mark.parametrize("ka,kw2,kb2", [(12, 4, 3), (20, 8, 5), (36, 4, 1)])
@pytest.mark.parametrize("n", [29, 65537])
def test_gram_tc5_tma_r1_width_4_mod_8(lib, torch_cuda, n, ka, kw2, kb2):
    """tcgen05 Gram Q^T [AQ | R] with the AQ part 4 columns past a multiple of
    8 (k = 4m, m odd) and R's rows 16-byte aligned (R = kb2 of kw2 columns):
    the TMA kernel takes AQ widened by 4 zero columns outside its tensor map
    and the reduction skips them."""
    torch = torch_cuda
    L = O.gen_rhs("normal", n, ka, 31).astype(np.float32)
    R1 = O.gen_rhs("normal", n, ka, 32).astype(np.float32)
    R2w = O.gen_rhs("normal", n, kw2, 33).astype(np.float32)
    want = O.port_gram(L.astype(np.float64),
                       np.hstack([R1, R2w[:, :kb2]]).astype(np.float64))
    d = {k_: dev(torch, a) for k_, a in dict(L=L, R1=R1, R2=R2w).items()}
    C = torch.zeros((ka, ka + kb2), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, 5, n, ptr(d["L"]), ka, ka, ptr(d["R1"]), ka, ka, ptr(d["R2"]), kw2,
                         kb2, ptr(C), ka + kb2, None)
    assert rc == 0
    assert relerr(host(C), want) <= 4e-6


@pytest.mark.parametrize("n", [31, 8191, 100003])
def test_gram_tc5_tma_subblocks(lib, torch_cuda, n):
    """tcgen05 Gram through TMA boxes on sub-blocks of wider arrays (row
    strides 48, 32 and 12; the tensor maps end at the block's last column, so
    the boxes zero-fill the rest): L = 40 of 48 columns, R1 = 24 of 32,
    R2 = 8 of 12."""
    torch = torch_cuda
    Lw = O.gen_rhs("normal", n, 48, 21).astype(np.float32)
    R1w = O.gen_rhs("normal", n, 32, 22).astype(np.float32)
    R2w = O.gen_rhs("normal", n, 12, 23).astype(np.float32)
    want = O.port_gram(Lw[:, :40].astype(np.float64),
                       np.hstack([R1w[:, :24], R2w[:, :8]]).astype(np.float64))
    d = {k_: dev(torch, a) for k_, a in dict(L=Lw, R1=R1w, R2=R2w).items()}
    C = torch.zeros((40, 32), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram(F32, 5, n, ptr(d["L"]), 48, 40, ptr(d["R1"]), 32, 24, ptr(d["R2"]), 12,
                         8, ptr(C), 32, None)
    assert rc == 0
    assert relerr(host(C), want) <= 4e-6
