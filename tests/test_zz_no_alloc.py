"""cacg_k_gram_noalloc: the Gram product for callers that cannot let the
library allocate device memory (their device memory belongs to their own
allocator, or an allocation could stall a latency-critical loop).  Its
split-K scratch is a fixed device array inside libcacg.so.

Checked through the C ABI against cacg_k_gram (which allocates a workspace),
within the tolerances the kernel tests use, on consecutive calls that reuse
the shared array; plus the empty case and the size limit.  Collected last
(file name) so that a stop-at-first-failure run has run every other test.
"""
import numpy as np
import pytest

import oracle as O
from gpu_util import dev, host, ptr, relerr

pytestmark = pytest.mark.gpu

F64, F32 = 0, 1


def _gram(lib, torch, fn, vt, variant, L, R1, R2):
    n, ka = L.shape
    kb1, kb2 = R1.shape[1], R2.shape[1]
    dL, d1, d2 = dev(torch, L), dev(torch, R1), dev(torch, R2)
    Cm = torch.full((ka, kb1 + kb2), np.nan, dtype=torch.float64, device="cuda")
    rc = fn(vt, variant, n, ptr(dL), ka, ka, ptr(d1), kb1, kb1, ptr(d2), kb2, kb2, ptr(Cm),
            kb1 + kb2, None)
    return rc, host(Cm)


@pytest.mark.parametrize("vt,variant,tol", [(F64, 1, 1e-12), (F64, 2, 1e-12), (F32, 0, 1e-10)])
def test_noalloc_matches_allocating_gram_twice(lib, torch_cuda, vt, variant, tol):
    torch = torch_cuda
    dt = np.float64 if vt == F64 else np.float32
    shapes = [(200000, 96, 96, 16), (30000, 64, 64, 8)]  # the first needs the chunk cap
    for call, (n, ka, kb1, kb2) in enumerate(shapes):
        L = O.gen_rhs("normal", n, ka, 10 + call).astype(dt)
        R1 = O.gen_rhs("normal", n, kb1, 20 + call).astype(dt)
        R2 = O.gen_rhs("normal", n, kb2, 30 + call).astype(dt)
        rc0, want = _gram(lib, torch, lib.cacg_k_gram, vt, variant, L, R1, R2)
        rc1, got = _gram(lib, torch, lib.cacg_k_gram_noalloc, vt, variant, L, R1, R2)
        assert rc0 == 0 and rc1 == 0
        assert np.isfinite(got).all()
        assert relerr(got, want) <= tol, (call, relerr(got, want))


def test_noalloc_empty_rows_give_zero(lib, torch_cuda):
    torch = torch_cuda
    L = O.gen_rhs("normal", 5000, 32, 1)
    R = O.gen_rhs("normal", 5000, 32, 2)
    rc, _ = _gram(lib, torch, lib.cacg_k_gram_noalloc, F64, 1, L, R, R[:, :4])
    assert rc == 0
    d = dev(torch, np.zeros((1, 32)))
    Cm = torch.full((32, 36), np.nan, dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram_noalloc(F64, 1, 0, ptr(d), 32, 32, ptr(d), 32, 32, ptr(d), 4, 4,
                                 ptr(Cm), 36, None)
    assert rc == 0
    assert (host(Cm) == 0.0).all()


def test_noalloc_rejects_oversized_shape(lib, torch_cuda):
    torch = torch_cuda
    d = dev(torch, np.zeros((8, 2048)))
    Cm = torch.zeros((2048, 2048), dtype=torch.float64, device="cuda")
    rc = lib.cacg_k_gram_noalloc(F64, 1, 8, ptr(d), 2048, 2048, ptr(d), 2048, 2048, None, 0, 0,
                                 ptr(Cm), 2048, None)
    assert rc == -1


@pytest.mark.parametrize("variant", [3, 4, 5, -1, 99])
def test_noalloc_refuses_other_variants(lib, torch_cuda, variant):
    """Only the CUDA-core variants (AUTO, FMA, DMMA) run from the fixed array;
    the tensor-core variants and unknown values are refused, not rerouted."""
    torch = torch_cuda
    L = O.gen_rhs("normal", 1000, 16, 1)
    rc, _ = _gram(lib, torch, lib.cacg_k_gram_noalloc, F64, variant, L, L, L[:, :4])
    assert rc == -6


def _runtime():
    """The CUDA runtime torch loaded (the default memory pool it reports is the
    device's, shared with libcacg.so's statically linked runtime)."""
    import ctypes as C

    for line in open("/proc/self/maps"):
        if "libcudart.so" in line:
            return C.CDLL(line.split()[-1])
    return C.CDLL("libcudart.so")


def test_noalloc_allocates_nothing(lib, torch_cuda):
    """The pool high-water mark stays at zero across the call (the allocating
    entry point's stream-ordered workspace comes from the same pool), and the
    device's free memory does not change."""
    import ctypes as C

    torch = torch_cuda
    rt = _runtime()
    L = O.gen_rhs("normal", 100000, 64, 3)
    R = O.gen_rhs("normal", 100000, 8, 4)
    dL, dR = dev(torch, L), dev(torch, R)
    Cm = torch.zeros((64, 72), dtype=torch.float64, device="cuda")
    args = (F64, 1, 100000, ptr(dL), 64, 64, ptr(dL), 64, 64, ptr(dR), 8, 8, ptr(Cm), 72, None)
    assert lib.cacg_k_gram(*args) == 0
    assert lib.cacg_k_gram_noalloc(*args) == 0  # first call: address lookup
    torch.cuda.synchronize()
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), torch.cuda.current_device()) == 0
    zero = C.c_uint64(0)
    USED_HIGH = 8  # cudaMemPoolAttrUsedMemHigh
    assert rt.cudaMemPoolSetAttribute(pool, USED_HIGH, C.byref(zero)) == 0
    free0, tot = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free0), C.byref(tot)) == 0
    for _ in range(2):
        assert lib.cacg_k_gram_noalloc(*args) == 0
    torch.cuda.synchronize()
    high = C.c_uint64(1)
    assert rt.cudaMemPoolGetAttribute(pool, USED_HIGH, C.byref(high)) == 0
    free1 = C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free1), C.byref(tot)) == 0
    assert high.value == 0
    assert free1.value == free0.value
    # and the result is still the allocating entry point's
    want = torch.zeros_like(Cm)
    args_w = args[:12] + (ptr(want),) + args[13:]
    assert lib.cacg_k_gram(*args_w) == 0
    assert relerr(host(Cm), host(want)) <= 1e-12
