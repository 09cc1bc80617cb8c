// cg_tma.cuh — the tensor memory accelerator and mbarrier operations of the staged kernels, as
// inline PTX (sm_90 and later: cp.async.bulk.tensor, mbarrier with transaction counts), and the
// host encoder of tensor maps (cuTensorMapEncodeTiled through the runtime's driver entry point,
// so the library links no driver library).
#pragma once

#include <cuda.h>  // CUtensorMap and its enums
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/chmy_gb300.h"  // cg_field

namespace cgtma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase of barrier b with the given parity; false when limit_ns ran out first.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try_wait(b, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (;;) {
        if (mbar_try_wait(b, parity)) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}
// One box of a 3D tensor map into shared memory; its bytes complete on barrier `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}


using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeFn encoder() {
    static const EncodeFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeFn) nullptr;
        }
        return reinterpret_cast<EncodeFn>(p);
    }();
    return fn;
}

// Elements between a field's first padded element and the 16-byte boundary at or before it;
// -1 when the field cannot have a tensor map (FP32 3D, 4-byte aligned, 16-byte row strides).
inline int map_offset(const cg_field& f) {
    if (f.dtype != CG_F32 || f.ndim != 3 || !f.data) return -1;
    const uintptr_t a = reinterpret_cast<uintptr_t>(f.data);
    if ((a & 3) != 0 || (f.stride[1] * 4) % 16 || (f.stride[2] * 4) % 16) return -1;
    return (int)((a & 15) >> 2);
}

// The tensor map of one FP32 field for boxes of w x h x 1 elements. Tensor coordinates start
// `xo` elements before the field's first padded element; ext (elements per dimension in those
// coordinates) may end before the padded extent, and box elements past it read as zero.
inline bool make_map_ext(const cg_field& f, int xo, const cuuint64_t ext[3], int w, int h, CUtensorMap* out) {
    const EncodeFn enc = encoder();
    if (!enc) return false;
    const uintptr_t a = reinterpret_cast<uintptr_t>(f.data);
    const cuuint64_t pad0 = (cuuint64_t)(f.n[0] + 4 * f.halo[0]) + (cuuint64_t)xo;
    const cuuint64_t pad1 = (cuuint64_t)(f.n[1] + 4 * f.halo[1]), pad2 = (cuuint64_t)(f.n[2] + 4 * f.halo[2]);
    if (ext[0] < 1 || ext[1] < 1 || ext[2] < 1 || ext[0] > pad0 || ext[1] > pad1 || ext[2] > pad2) return false;
    const cuuint64_t st1 = (cuuint64_t)f.stride[1] * 4, st2 = (cuuint64_t)f.stride[2] * 4;
    if ((cuuint64_t)f.stride[1] < pad0 || st2 < st1 * pad1) return false;
    const cuuint64_t strides[2] = {st1, st2};
    const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)h, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    void* base = reinterpret_cast<void*>(a - (uintptr_t)xo * 4);
    return enc(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, ext, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace cgtma
