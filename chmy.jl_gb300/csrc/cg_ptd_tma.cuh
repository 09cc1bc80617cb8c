// cg_ptd_tma.cuh — the fused 3D PT-diffusion iteration (update_q! + update_C!, the arithmetic of
// ptd_march3d_kernel) with its inputs staged by the tensor memory accelerator.
//
// ptd_march3d_kernel waits on its own loads: each warp has one plane of loads in flight, and
// most of its issue cycles stall on them. Here one thread of the block streams whole z-planes
// of the block's tile — the six input arrays (C, D, q_x, q_y, q_z, C_old) over the tile's rows
// with one halo row on each side and 40 columns — into a ring of kStages planes in shared
// memory with cp.async.bulk.tensor, kStages - 2 planes ahead of the two the warps read. Each
// ring slot has a `full` mbarrier (the copies' bytes arrive) and an `empty` mbarrier (every warp
// has read the plane). The warps compute exactly what ptd_march3d_kernel computes, from shared
// memory instead of global loads, so the results are bitwise the same. Every wait is bounded by
// %globaltimer: a wait that runs out sets the error flag and the block stops; the producing
// thread then waits, again bounded, for its copies still in flight before the block exits.
//
// Layout requirements (checked on the host): FP32, every array's rows 16-byte aligned with
// strides that are multiples of 16 bytes, and a shared row and plane stride (the fused kernel's
// condition). The tensor map of an array starts at its first padded element rounded down to
// 16 bytes (xo elements before it) and covers exactly its padded extent, so no copy reads past
// the allocation; columns beyond it read as zero and are never used.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums (the encoder is reached through the runtime)

namespace ptdt {

constexpr int kCols = 40;    // box width: 32 tile columns, the x halos and the 16-byte alignment slack
constexpr int kStages = 4;   // ring slots: the two planes in use and two in flight
constexpr int kArrays = 6;   // box order
enum { A_C = 0, A_D = 1, A_QX = 2, A_QY = 3, A_QZ = 4, A_CO = 5 };

struct Maps {
    CUtensorMap m[kArrays];
};
// Elements between each array's map origin (16-byte aligned) and its first padded element.
struct XO {
    int v[kArrays];
};

template <int NW>
struct Geom {
    static constexpr int rows = NW + 2;
    static constexpr int box_floats = kCols * rows;
    static constexpr int box_bytes = (box_floats * 4 + 127) / 128 * 128;  // each box 128-byte aligned
    static constexpr int stage_bytes = kArrays * box_bytes;
    static constexpr unsigned tx_bytes = kArrays * box_floats * 4;
    // the ring, the 2 x kStages barriers and 128 bytes to align the ring's start
    static constexpr int smem_bytes = kStages * stage_bytes + 2 * kStages * 8 + 128;
};

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

}  // namespace ptdt

// The TMA-fed fused iteration. Block = NW warps over a tile of 32 x NW (i, j) columns and one z
// segment; plane m of the ring is logical plane ks - 1 + m (tensor z = ks + m), box rows are the
// logical rows j0 - 1 .. j0 + NW (tensor y = j0 ...), box column c is tensor x = i0 + c, i.e.
// logical i0 - 1 - xo + c for an array whose map starts xo elements before its first element.
template <int NW, int MINB>
__global__ void __launch_bounds__(32 * NW, MINB)
    ptd_tma_kernel(const __grid_constant__ ptdt::Maps maps, const PDM<float> f, const ptdt::XO xo, int e0, int e1, int e2,
                   int ntx, int nty, int seg_len, unsigned long long limit_ns, int* err) {
    using namespace cgk;
    using namespace ptdt;
    using G = Geom<NW>;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(128) unsigned char smdyn[];
    // the ring starts on a 128-byte boundary of the shared window (the copies' destinations)
    unsigned char* smraw = smdyn + ((128u - (smem_u32(smdyn) & 127u)) & 127u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smraw + kStages * G::stage_bytes);
    uint64_t* empty = full + kStages;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int tx = b % ntx, ty = (b / ntx) % nty, seg = b / (ntx * nty);
    const int ks = seg * seg_len;
    if (ks > e2) return;  // whole block, before any barrier exists
    const int ke = min(ks + seg_len - 1, e2);
    const int i0 = tx * 32, j0 = ty * NW;
    const int i = i0 + lane, j = j0 + w;
    const bool row = j <= e1;  // warp-uniform: the row is in the launch range
    PDFlags fl;
    fl.cx = row && i <= e0;
    fl.lx = row && i <= e0 + 1;
    fl.yu = j + 1 <= e1;
    fl.h0 = lane == 0 && fl.cx;
    fl.h31c = lane == 31 && row && i + 1 <= e0;
    fl.h31q = lane == 31 && row && i + 1 <= e0 + 1;
    const int nplanes = ke - ks + 3;  // planes ks-1 .. ke+1
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NW);
        }
        mbar_fence_init();
    }
    __syncthreads();
    static_assert((kStages & (kStages - 1)) == 0, "the ring's slot index is a mask");
    auto slot = [&](int m) { return smraw + (m & (kStages - 1)) * G::stage_bytes; };
    auto issue = [&](int m) {
        unsigned char* dst = slot(m);
        uint64_t* bar = &full[m & (kStages - 1)];
        mbar_expect_tx(bar, G::tx_bytes);
        for (int a = 0; a < kArrays; ++a) tma_load_3d(dst + a * G::box_bytes, &maps.m[a], i0, j0, ks + m, bar);
    };
    int issued = -1, waited = -1;  // producer's bookkeeping (thread 0)
    if (threadIdx.x == 0) {
        const int first = nplanes < kStages ? nplanes : kStages;
        for (int m = 0; m < first; ++m) issue(m);
        issued = first - 1;
    }
    // the lane's element of array a, row r0 = w + 1 of the box, as a float offset into a slot;
    // a neighbour is a compile-time displacement (dr rows, dc columns) from it
    const int r0 = w + 1;
    constexpr int SF = G::stage_bytes / 4, BF = G::box_bytes / 4;
    int col[kArrays];
#pragma unroll
    for (int a = 0; a < kArrays; ++a) col[a] = a * BF + r0 * kCols + lane + 1 + xo.v[a];
    const float* ring = reinterpret_cast<const float*>(smraw);
    auto V = [&](int m, int a, int dr, int dc) -> float {
        return ring[(m & (kStages - 1)) * SF + col[a] + dr * kCols + dc];
    };
    bool ok = mbar_wait(&full[0], 0, limit_ns) && mbar_wait(&full[1 & (kStages - 1)], (1 / kStages) & 1, limit_ns);
    // every decision to stop is taken by the whole warp (shuffles below need all 32 lanes)
    ok = __all_sync(FULL, ok);
    waited = ok ? 1 : -1;
    // prologue: the new flux of plane ks's lower z face (C and D of planes ks-1 and ks)
    float qzl = 0.f;
    if (ok && fl.cx) qzl = pd_face(V(1, A_QZ, 0, 0), V(0, A_D, 0, 0), V(1, A_D, 0, 0), V(0, A_C, 0, 0), V(1, A_C, 0, 0),
                                   f.idx[2], f.om);
    __syncwarp();
    if (ok && lane == 0) mbar_arrive(&empty[0]);
    int o = i + j * f.s1 + ks * f.s2;
    for (int t = 0; ok && t <= ke - ks; ++t, o += f.s2) {
        const int k = ks + t;
        const int mc = t + 1, mn = t + 2;  // planes k and k+1
        // refill the slot of plane t (every warp released it) with plane t + kStages
        if (threadIdx.x == 0 && t + kStages < nplanes) {
            if (mbar_wait(&empty[t & (kStages - 1)], (t / kStages) & 1, limit_ns)) {
                issue(t + kStages);
                issued = t + kStages;
            } else {
                ok = false;
            }
        }
        if (ok && !mbar_wait(&full[mn & (kStages - 1)], (mn / kStages) & 1, limit_ns)) ok = false;
        ok = __all_sync(FULL, ok);
        if (!ok) break;
        waited = mn;
        if (row) {
            // ptd_march3d_kernel's step on the values it loads (C and D of plane k at the point,
            // its x, y neighbours and plane k+1; the stored fluxes; C_old), read from the ring.
            // Values a guard leaves unused there are unused here too.
            const float c = V(mc, A_C, 0, 0), d = V(mc, A_D, 0, 0);
            const float qxs = fl.lx ? V(mc, A_QX, 0, 0) : 0.f;
            const float qxl = fl.cx ? pd_face(qxs, V(mc, A_D, 0, -1), d, V(mc, A_C, 0, -1), c, f.idx[0], f.om) : qxs;
            float qxu = __shfl_down_sync(FULL, qxl, 1);
            if (lane == 31) {
                const float hq = fl.h31q ? V(mc, A_QX, 0, 1) : 0.f;
                qxu = fl.h31c ? pd_face(hq, d, V(mc, A_D, 0, 1), c, V(mc, A_C, 0, 1), f.idx[0], f.om) : hq;
            }
            if (fl.cx) {
                const float qyl = pd_face(V(mc, A_QY, 0, 0), V(mc, A_D, -1, 0), d, V(mc, A_C, -1, 0), c, f.idx[1], f.om);
                const float qys = V(mc, A_QY, 1, 0);
                const float qyu = fl.yu ? pd_face(qys, d, V(mc, A_D, 1, 0), c, V(mc, A_C, 1, 0), f.idx[1], f.om) : qys;
                const float qzs = V(mn, A_QZ, 0, 0);
                const float qzu = k + 1 <= e2 ? pd_face(qzs, d, V(mn, A_D, 0, 0), c, V(mn, A_C, 0, 0), f.idx[2], f.om) : qzs;
                float dv = rmul(rsub(qxu, qxl), f.idx[0]);
                dv = radd(dv, rmul(rsub(qyu, qyl), f.idx[1]));
                dv = radd(dv, rmul(rsub(qzu, qzl), f.idx[2]));
                const float rr = rsub(rmul(-rsub(c, V(mc, A_CO, 0, 0)), f.inv_dt), dv);
                f.Cn[o] = radd(c, rmul(rr, f.dtc));
                f.qn[0][o] = qxl;
                f.qn[1][o] = qyl;
                f.qn[2][o] = qzl;
                qzl = qzu;
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[mc & (kStages - 1)]);
    }
    if (!ok) {
        atomicExch(err, 1);
        // the producing thread's copies still in flight complete before the block's shared
        // memory goes away (bounded; they complete unless the copy itself failed)
        if (threadIdx.x == 0)
            for (int m = waited + 1; m <= issued; ++m) mbar_wait(&full[m & (kStages - 1)], (m / kStages) & 1, limit_ns);
    }
}

namespace ptdt {

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

// The tensor map of one FP32 field for boxes of kCols x rows x 1; false when its layout does not
// allow one (16-byte row alignment and strides).
inline bool make_map(const cg_field& f, int rows, CUtensorMap* out, int* xo) {
    const EncodeFn enc = encoder();
    if (!enc || f.dtype != CG_F32 || f.ndim != 3 || !f.data) return false;
    const uintptr_t a = reinterpret_cast<uintptr_t>(f.data);
    if ((a & 3) != 0) return false;
    *xo = (int)((a & 15) >> 2);
    const cuuint64_t ext0 = (cuuint64_t)(f.n[0] + 4 * f.halo[0]) + (cuuint64_t)*xo;
    const cuuint64_t ext1 = (cuuint64_t)(f.n[1] + 4 * f.halo[1]), ext2 = (cuuint64_t)(f.n[2] + 4 * f.halo[2]);
    const cuuint64_t st1 = (cuuint64_t)f.stride[1] * 4, st2 = (cuuint64_t)f.stride[2] * 4;
    if (st1 % 16 || st2 % 16 || (cuuint64_t)f.stride[1] < ext0 || st2 < st1 * ext1) return false;
    const cuuint64_t dims[3] = {ext0, ext1, ext2};
    const cuuint64_t strides[2] = {st1, st2};
    const cuuint32_t box[3] = {(cuuint32_t)kCols, (cuuint32_t)rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    void* base = reinterpret_cast<void*>(a - (uintptr_t)(*xo) * 4);
    return enc(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The six maps of one launch direction (inputs C, q read; D and C_old shared by both).
inline bool make_maps(const cg_field& C, const cg_field* q, const cg_field& D, const cg_field& Co, int rows, Maps* m,
                      XO* xo) {
    return make_map(C, rows, &m->m[A_C], &xo->v[A_C]) && make_map(D, rows, &m->m[A_D], &xo->v[A_D]) &&
           make_map(q[0], rows, &m->m[A_QX], &xo->v[A_QX]) && make_map(q[1], rows, &m->m[A_QY], &xo->v[A_QY]) &&
           make_map(q[2], rows, &m->m[A_QZ], &xo->v[A_QZ]) && make_map(Co, rows, &m->m[A_CO], &xo->v[A_CO]);
}

}  // namespace ptdt

// Maps for both ping-pong directions of a fused run, for the two block heights of the TMA
// variants (8 and 16 rows), and the device error flag the kernel raises on a wait that ran out.
struct PdTma {
    bool ok = false;
    ptdt::Maps ab8, ba8, ab16, ba16;
    ptdt::XO xab, xba;
    int* err = nullptr;
};

inline PdTma make_pd_tma(const cg_field& Ca, const cg_field* qa, const cg_field& Cb, const cg_field* qb, const cg_field& D,
                         const cg_field& Co, int* err) {
    PdTma t;
    t.err = err;
    ptdt::XO x2;
    t.ok = err && ptdt::make_maps(Ca, qa, D, Co, 10, &t.ab8, &t.xab) && ptdt::make_maps(Cb, qb, D, Co, 10, &t.ba8, &t.xba) &&
           ptdt::make_maps(Ca, qa, D, Co, 18, &t.ab16, &x2) && ptdt::make_maps(Cb, qb, D, Co, 18, &t.ba16, &x2);
    return t;
}
