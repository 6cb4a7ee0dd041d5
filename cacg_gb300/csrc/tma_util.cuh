// tma_util.cuh -- host-side TMA descriptors (cuTensorMapEncodeTiled through
// the runtime's driver entry point, so libcacg does not link libcuda) and
// the device-side 2-D tiled load with mbarrier completion.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cacg {

inline PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// FP32 2-D map: `inner` elements per row (contiguous), `outer` rows
// `row_bytes` apart; box box_in x box_out; zero fill outside the tensor.
inline bool tma_encode_2d(CUtensorMap *m, const void *base, uint64_t inner, uint64_t outer,
                          uint64_t row_bytes, uint32_t box_in, uint32_t box_out,
                          CUtensorMapSwizzle swizzle, CUtensorMapL2promotion promo) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = tma_encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_in, box_out};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides, box,
              es, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, promo,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

#ifdef __CUDACC__
__device__ __forceinline__ unsigned tma_smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

// arrive on *bar announcing `bytes` of transactions for the current phase
__device__ __forceinline__ void tma_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile(
        "{\n"
        ".reg .b64 st;\n"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n"
        "}\n" ::"r"(tma_smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

// 2-D tiled TMA load of the box at (x, y) (elements; x innermost) into dst
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];\n" ::"r"(tma_smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(tma_smem_u32(bar))
        : "memory");
}

// 2-D tiled TMA store of the box at (x, y) from src (rows outside the tensor
// are not written); completion is tracked by the calling thread's bulk groups
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y,
                                             const void *src) {
    asm volatile(
        "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(x), "r"(y), "r"(tma_smem_u32(src))
        : "memory");
}
__device__ __forceinline__ void tma_store_commit() {
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}
// the shared-memory sources of this thread's committed stores have been read
__device__ __forceinline__ void tma_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
}
// this thread's committed stores are complete
__device__ __forceinline__ void tma_store_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}
#endif

}  // namespace cacg
