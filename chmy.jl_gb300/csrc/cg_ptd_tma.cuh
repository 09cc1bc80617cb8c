// cg_ptd_tma.cuh — the fused 3D PT-diffusion iteration (update_q! + update_C!, the arithmetic of
// ptd_march3d_kernel) with its inputs staged by the tensor memory accelerator.
//
// ptd_march3d_kernel waits on its own loads: each warp has one plane of loads in flight, and
// most of its issue cycles stall on them. Here one thread of the block streams whole z-planes
// of the block's tile — the six input arrays (C, D, q_x, q_y, q_z, C_old) over the tile's rows
// with one halo row where it is read — into a ring of S planes in shared memory with
// cp.async.bulk.tensor, S - 2 planes ahead of the two the warps read. Each
// ring slot has a `full` mbarrier (the copies' bytes arrive) and an `empty` mbarrier (every warp
// has read the plane). The warps compute exactly what ptd_march3d_kernel computes, from shared
// memory instead of global loads, so the results are bitwise the same. Every wait is bounded by
// %globaltimer: a wait that runs out sets the error flag and the block stops; the producing
// thread then waits, again bounded, for its copies still in flight before the block exits.
//
// Layout requirements (checked on the host): FP32, 4-byte aligned arrays with row and plane
// strides that are multiples of 16 bytes, and a shared row and plane stride (the fused kernel's
// condition). The tensor map of an array starts at its first padded element rounded down to
// 16 bytes (xo elements before it) and covers exactly its padded extent, so no copy reads past
// the allocation; box elements beyond it read as zero and are never used.
#pragma once

#include "cg_tma.cuh"

namespace ptdt {

using namespace cgtma;

constexpr int kCols = 40;    // box width: 32 tile columns, the x halos and the 16-byte alignment slack
constexpr int kArrays = 6;   // box order
enum { A_C = 0, A_D = 1, A_QX = 2, A_QY = 3, A_QZ = 4, A_CO = 5 };

struct Maps {
    CUtensorMap m[kArrays];
};
// The box of each array in one launch. An array's box covers just the columns and rows the
// iteration reads from it: C and D the tile's 32 columns with one halo column on each side and
// one halo row on each side; q_x the columns and the upper x halo, q_y the rows and the upper y
// halo row; q_z and C_old the tile alone. Along x the box starts on a 16-byte boundary at or
// before the first column it needs and has a width that is a multiple of 4 elements.
struct Boxes {
    int x0[kArrays];   // box start along x in tensor coordinates, relative to the tile's i0
    int y0[kArrays];   // box start along y relative to j0 (tensor y = logical y + 1): 0 or 1
    int w[kArrays];    // box width (floats)
    int cb[kArrays];   // box column of the lane's column = lane + cb
    int off[kArrays];  // the box's float offset in a ring slot (128-byte aligned)
    int sf;            // floats per ring slot
    unsigned tx;       // bytes one slot's copies deliver
};

// Shared memory a block's ring needs: S slots of sf floats, the 2 x S barriers and 128 bytes to
// align the ring's start.
inline int smem_bytes(int S, int sf) { return S * sf * 4 + 2 * S * 8 + 128; }
// The same for boxes all kCols wide and NW + 2 rows high, the largest a launch can need.
template <int NW, int S>
constexpr int max_smem_bytes() {
    return S * kArrays * ((kCols * (NW + 2) * 4 + 127) / 128 * 128) + 2 * S * 8 + 128;
}
// Rows of array a's box for blocks of NW rows.
__host__ __device__ constexpr int box_rows(int a, int nw) {
    return (a == A_C || a == A_D) ? nw + 2 : (a == A_QY ? nw + 1 : nw);
}

}  // namespace ptdt

// The TMA-fed fused iteration. Block = NW warps over a tile of 32 x NW (i, j) columns and one z
// segment; plane m of the ring is logical plane ks - 1 + m (tensor z = ks + m); array a's box in
// a slot starts at tensor (i0 + x0, j0 + y0) (Boxes).
template <int NW, int MINB, int S>
__global__ void __launch_bounds__(32 * NW, MINB)
    ptd_tma_kernel(const __grid_constant__ ptdt::Maps maps, const PDM<float> f, const ptdt::Boxes bx, int e0, int e1, int e2,
                   int ntx, int nty, int seg_len, unsigned long long limit_ns, int withhold, int* err) {
    using namespace cgk;
    using namespace ptdt;
    using namespace cgtma;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(128) unsigned char smdyn[];
    // the ring starts on a 128-byte boundary of the shared window (the copies' destinations)
    unsigned char* smraw = smdyn + ((128u - (smem_u32(smdyn) & 127u)) & 127u);
    static_assert(S >= 3 && (S & (S - 1)) == 0, "the ring holds two planes in use and one in flight; its index is a mask");
    uint64_t* full = reinterpret_cast<uint64_t*>(smraw + (size_t)S * bx.sf * 4);
    uint64_t* empty = full + S;
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
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NW);
        }
        mbar_fence_init();
    }
    __syncthreads();
    float* ring = reinterpret_cast<float*>(smraw);
    auto issue = [&](int m) {
        if (m == withhold) return;  // a test's withheld plane: its waits run out
        float* dst = ring + (m & (S - 1)) * bx.sf;
        uint64_t* bar = &full[m & (S - 1)];
        mbar_expect_tx(bar, bx.tx);
        for (int a = 0; a < kArrays; ++a)
            tma_load_3d(dst + bx.off[a], &maps.m[a], i0 + bx.x0[a], j0 + bx.y0[a], ks + m, bar);
    };
    int issued = -1, waited = -1;  // producer's bookkeeping (thread 0)
    if (threadIdx.x == 0) {
        const int first = nplanes < S ? nplanes : S;
        for (int m = 0; m < first; ++m) issue(m);
        issued = first - 1;
    }
    // the lane's element of array a in the warp's row, as a float offset into a slot (the row
    // j = j0 + w is box row w + 1 - y0); a neighbour is dr rows and dc columns away
    int col[kArrays];
#pragma unroll
    for (int a = 0; a < kArrays; ++a) col[a] = bx.off[a] + (w + 1 - bx.y0[a]) * bx.w[a] + lane + bx.cb[a];
    auto V = [&](int m, int a, int dr, int dc) -> float {
        return ring[(m & (S - 1)) * bx.sf + col[a] + dr * bx.w[a] + dc];
    };
    bool ok = mbar_wait(&full[0], 0, limit_ns) && mbar_wait(&full[1 & (S - 1)], (1 / S) & 1, limit_ns);
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
        // refill the slot of plane t (every warp released it) with plane t + S
        if (threadIdx.x == 0 && t + S < nplanes) {
            if (mbar_wait(&empty[t & (S - 1)], (t / S) & 1, limit_ns)) {
                issue(t + S);
                issued = t + S;
            } else {
                ok = false;
            }
        }
        if (ok && !mbar_wait(&full[mn & (S - 1)], (mn / S) & 1, limit_ns)) ok = false;
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
        if (lane == 0) mbar_arrive(&empty[mc & (S - 1)]);
    }
    if (!ok) {
        atomicExch(err, 1);
        // the producing thread's copies still in flight complete before the block's shared
        // memory goes away (bounded; they complete unless the copy itself failed)
        if (threadIdx.x == 0)
            for (int m = waited + 1; m <= issued; ++m)
                if (m != withhold) mbar_wait(&full[m & (S - 1)], (m / S) & 1, limit_ns);
    }
}

namespace ptdt {

// The tensor map of one field for boxes of w x h x 1 elements; it covers exactly the field's
// padded extent, from `xo` elements before its first padded element.
inline bool make_map(const cg_field& f, int xo, int w, int h, CUtensorMap* out) {
    const cuuint64_t ext[3] = {(cuuint64_t)(f.n[0] + 4 * f.halo[0]) + (cuuint64_t)xo, (cuuint64_t)(f.n[1] + 4 * f.halo[1]),
                               (cuuint64_t)(f.n[2] + 4 * f.halo[2])};
    return make_map_ext(f, xo, ext, w, h, out);
}

// Maps and boxes of one launch direction (inputs C, q read; D and C_old shared by both) for
// blocks of nw rows. Array a needs the logical columns i0 + lo .. i0 + hi of a tile starting at
// column i0 (a multiple of 32), i.e. tensor columns i0 + lo + 1 + xo .. i0 + hi + 1 + xo.
inline bool make_maps(const cg_field& C, const cg_field* q, const cg_field& D, const cg_field& Co, int nw, Maps* m,
                      Boxes* bx) {
    const cg_field* fs[kArrays] = {&C, &D, &q[0], &q[1], &q[2], &Co};
    const int lo[kArrays] = {-1, -1, 0, 0, 0, 0}, hi[kArrays] = {32, 32, 32, 31, 31, 31};
    int off = 0;
    unsigned tx = 0;
    for (int a = 0; a < kArrays; ++a) {
        const int xo = map_offset(*fs[a]);
        if (xo < 0) return false;
        const int first = lo[a] + 1 + xo, last = hi[a] + 1 + xo;
        const int x0 = first & ~3;
        const int w = (last - x0 + 1 + 3) & ~3;
        const int h = box_rows(a, nw);
        if (w > kCols || !make_map(*fs[a], xo, w, h, &m->m[a])) return false;
        bx->x0[a] = x0;
        bx->y0[a] = (a == A_C || a == A_D) ? 0 : 1;
        bx->w[a] = w;
        bx->cb[a] = 1 + xo - x0;
        bx->off[a] = off;
        off += ((w * h * 4 + 127) / 128) * 32;
        tx += (unsigned)(w * h * 4);
    }
    bx->sf = off;
    bx->tx = tx;
    return true;
}

}  // namespace ptdt

// Maps and boxes for both ping-pong directions of a fused run, for the two block heights of the
// TMA variants (8 and 16 rows), and the device error flag the kernel raises on a wait that ran
// out.
constexpr int kPdHeights = 4;
constexpr int kPdHeight[kPdHeights] = {8, 16, 20, 24};  // block rows of the TMA variants

struct PdTma {
    bool ok = false;
    ptdt::Maps ab[kPdHeights], ba[kPdHeights];
    ptdt::Boxes bab[kPdHeights], bba[kPdHeights];
    int* err = nullptr;
};

inline PdTma make_pd_tma(const cg_field& Ca, const cg_field* qa, const cg_field& Cb, const cg_field* qb, const cg_field& D,
                         const cg_field& Co, int* err) {
    PdTma t;
    t.err = err;
    t.ok = err != nullptr;
    for (int h = 0; h < kPdHeights && t.ok; ++h)
        t.ok = ptdt::make_maps(Ca, qa, D, Co, kPdHeight[h], &t.ab[h], &t.bab[h]) &&
               ptdt::make_maps(Cb, qb, D, Co, kPdHeight[h], &t.ba[h], &t.bba[h]);
    return t;
}
