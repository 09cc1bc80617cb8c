// cg_ptdiff.cu — pseudo-transient variable-coefficient diffusion (implicit step solved by
// damped PT iterations; flux in Chmy's ∂k∂ form, src/GridOperators/partial_derivatives.jl:14-21).
#include "cg_common.cuh"

#include <cmath>


namespace {

template <class T>
struct PV {
    DF<T> C, Co, D, q[3], R;
    int has_R;
    T idx[3];
    T om, inv_dt, dtc;
};

template <class T>
PV<T> make_pv(const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    PV<T> v;
    std::memset(&v, 0, sizeof(v));
    v.C = cg_view<T>(f->C);
    v.Co = cg_view<T>(f->C_old);
    v.D = cg_view<T>(f->D);
    for (int d = 0; d < g->ndim; ++d) v.q[d] = cg_view<T>(f->q[d]);
    if (cg_present(f->R)) {
        v.R = cg_view<T>(f->R);
        v.has_R = 1;
    }
    for (int d = 0; d < 3; ++d) v.idx[d] = (T)g->inv_spacing[d];
    v.om = (T)p->omega_q;
    v.inv_dt = T(1) / (T)p->dt;
    v.dtc = (T)p->dtau_C;
    return v;
}

template <int ND>
inline dim3 range_grid(const cg_grid* g, dim3 block) {
    return dim3(cg_div_up(g->n[0] + 2, block.x), ND > 1 ? cg_div_up(g->n[1] + 2, block.y) : 1, ND > 2 ? g->n[2] + 2 : 1);
}
template <int ND>
inline dim3 block_for() {
    return ND == 1 ? dim3(256, 1) : dim3(32, 8);
}

// q_d += (-(lerp(D -> face_d) * ∂_d C) - q_d) * omega_q at I in [0, n+1]^N
template <class T, int ND>
__global__ void ptdiff_q_kernel(const PV<T> v, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const T c = v.C(i, j, k), dc = v.D(i, j, k);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const int di = d == 0, dj = d == 1, dk = d == 2;
        const T dl = v.D(i - di, j - dj, k - dk);
        const T Df = fma(T(0.5), dc - dl, dl);
        const T gC = (c - v.C(i - di, j - dj, k - dk)) * v.idx[d];
        const T qo = v.q[d](i, j, k);
        v.q[d](i, j, k) = qo + (-(Df * gC) - qo) * v.om;
    }
}

// R = -(C - C_old)/dt - divg(q); C += R dtau_C at I in [0, n+1]^N
template <class T, int ND>
__global__ void ptdiff_C_kernel(const PV<T> v, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    T dv = (v.q[0](i + 1, j, k) - v.q[0](i, j, k)) * v.idx[0];
    if (ND > 1) dv = dv + (v.q[1](i, j + 1, k) - v.q[1](i, j, k)) * v.idx[1];
    if (ND > 2) dv = dv + (v.q[2](i, j, k + 1) - v.q[2](i, j, k)) * v.idx[2];
    const T c = v.C(i, j, k);
    const T r = -(c - v.Co(i, j, k)) * v.inv_dt - dv;
    if (v.has_R) v.R(i, j, k) = r;
    v.C(i, j, k) = c + r * v.dtc;
}

int check_ptdiff(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    int rc = cg_check_grid(ctx, g);
    if (rc) return rc;
    if (!f || !p) return cg_fail(ctx, CG_ERR_ARG, "ptdiff: NULL argument");
    const int dt = f->C.dtype;
    if ((rc = cg_check_field(ctx, g, f->C, dt, 0, "C"))) return rc;
    if ((rc = cg_check_field(ctx, g, f->C_old, dt, 0, "C_old"))) return rc;
    if ((rc = cg_check_field(ctx, g, f->D, dt, 0, "D"))) return rc;
    for (int d = 0; d < g->ndim; ++d)
        if ((rc = cg_check_field(ctx, g, f->q[d], dt, 1 << d, "q"))) return rc;
    if (cg_present(f->R) && (rc = cg_check_field(ctx, g, f->R, dt, 0, "R"))) return rc;
    if (!(p->dt > 0)) return cg_fail(ctx, CG_ERR_ARG, "ptdiff: dt must be > 0");
    return CG_OK;
}

// Bytes from the first to the last element of the padded field (pitched rows included).
size_t padded_bytes(const cg_field& f) {
    size_t span = 1;
    for (int d = 0; d < f.ndim; ++d) span += (size_t)(f.n[d] + 4 * f.halo[d] - 1) * (size_t)f.stride[d];
    return span * (f.dtype == CG_F64 ? 8 : 4);
}

template <class T, int ND>
int launch_q(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p,
             dim3 b = block_for<ND>()) {
    ptdiff_q_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(make_pv<T>(g, f, p), g->n[0] + 1,
                                                                         ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int launch_C(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p,
             dim3 b = block_for<ND>()) {
    ptdiff_C_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(make_pv<T>(g, f, p), g->n[0] + 1,
                                                                         ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// Block shapes of the flux and update kernels of a PT run over this field set (tune_block;
// cached per grid, precision and layout; 1D keeps 256 threads). The kernels update q and C in
// place and write R, so the candidates run on copies of those fields in a temporary
// allocation, released before the run's graph is captured; the caller's fields are untouched.
template <class T, int ND>
int ptdiff_blocks(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p, dim3* bq,
                  dim3* bc) {
    *bq = *bc = block_for<ND>();
    if (ND == 1) return CG_OK;
    dim3 forced;
    if (cg_block_forced(&forced)) {
        *bq = *bc = forced;
        return CG_OK;
    }
    if (!cg_autotune_enabled()) return CG_OK;
    std::string base = "ptdiff_blocks";
    cg_key_add(base, *g);
    cg_key_add(base, (int)sizeof(T));
    cg_key_add(base, f->C.stride);
    cg_key_add(base, f->q[0].stride);
    cg_key_add(base, (int)cg_present(f->R));
    cg_key_add(base, ctx->num_sms);
    const std::string kq = base + "q", kc = base + "C";
    cg_tune_cfg c1{0, 0}, c2{0, 0};
    if (cg_tune_lookup(kq, &c1) && cg_tune_lookup(kc, &c2)) {
        *bq = dim3((unsigned)c1.seg, (unsigned)c1.variant);
        *bc = dim3((unsigned)c2.seg, (unsigned)c2.variant);
        return CG_OK;
    }
    cg_ptdiff_fields c = *f;
    cg_field* upd[5];
    int nu = 0;
    upd[nu++] = &c.C;
    for (int d = 0; d < ND; ++d) upd[nu++] = &c.q[d];
    if (cg_present(c.R)) upd[nu++] = &c.R;
    size_t off[5], total = 0;
    for (int a = 0; a < nu; ++a) {
        off[a] = total;
        total += (padded_bytes(*upd[a]) + 255) & ~(size_t)255;
    }
    char* tmp = nullptr;
    if (cudaMalloc(&tmp, total) != cudaSuccess) {
        cudaGetLastError();
        return CG_OK;  // no room to time the candidates: the default shape
    }
    for (int a = 0; a < nu; ++a) {
        const cudaError_t e = cudaMemcpyAsync(tmp + off[a], upd[a]->data, padded_bytes(*upd[a]), cudaMemcpyDeviceToDevice,
                                              ctx->stream);
        if (e != cudaSuccess) {
            cudaFree(tmp);
            return cg_fail(ctx, CG_ERR_CUDA, "ptdiff block tuning: %s", cudaGetErrorString(e));
        }
        upd[a]->data = tmp + off[a];
    }
    const PV<T> v = make_pv<T>(g, &c, p);
    const int e0 = g->n[0] + 1, e1 = ND > 1 ? g->n[1] + 1 : 0;
    *bq = cgk::tune_block("ptdiff update_q", kq,
                          [&](dim3 b) {
                              ptdiff_q_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(v, e0, e1);
                              return cudaGetLastError();
                          },
                          ctx->stream);
    *bc = cgk::tune_block("ptdiff update_C", kc,
                          [&](dim3 b) {
                              ptdiff_C_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(v, e0, e1);
                              return cudaGetLastError();
                          },
                          ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(tmp);
    return CG_OK;
}

#define PDISPATCH(fn, dtype, nd, ...)                                                                     \
    ((dtype) == CG_F64 ? ((nd) == 1 ? fn<double, 1>(__VA_ARGS__)                                         \
                                    : (nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__)) \
                       : ((nd) == 1 ? fn<float, 1>(__VA_ARGS__)                                          \
                                    : (nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

// ---- fused 3D PT iteration: update_q! + update_C! in one z-marching pass ---------------------
//
// One launch computes, for every cell I of the launch range [0, n+1]^3, the new flux on its
// three lower faces and the new C. It reads the `in` buffers (C, q) and writes the `out`
// buffers (ping-pong), so every value it reads is the previous iteration's. A warp holds 32
// consecutive x columns of one y row and marches up a segment of z planes:
// - x: the lower face of column i needs C and D of column i-1, from the lane below (lane 0
//   loads them). Its upper face is the next lane's lower face; lane 31 computes its own.
// - y: the row computes both faces. The upper one is the next row's lower face, recomputed
//   with the same operations, so it rounds identically.
// - z: the upper face of plane k is the lower face of plane k+1, carried in a register.
// A face at index n+2 lies beyond the two-kernel form's flux launch range and keeps its stored
// value. Every operation rounds once, in the oracle's order, so the result equals the
// oracle's update_q! followed by update_C!, bit for bit.
template <class T>
struct PDM {
    T* C;   // in (each pointer at logical (0, 0, 0))
    T* q[3];
    T* Cn;  // out
    T* qn[3];
    const T* Co;
    const T* D;
    int s1, s2;  // row and plane strides shared by every array
    T idx[3], om, inv_dt, dtc;
};

// q + (-(lerp(D) dC) - q) omega_q on the face between cells a (lower) and b (upper)
template <class T>
__device__ __forceinline__ T pd_face(T qo, T da, T db, T ca, T cb, T idx, T om) {
    using namespace cgk;
    const T Df = rfma(T(0.5), rsub(db, da), da);
    const T gC = rmul(rsub(cb, ca), idx);
    return radd(qo, rmul(rsub(-rmul(Df, gC), qo), om));
}

// The loads of plane k for the thread at element offset o: its x flux, the y neighbours' C
// and D with both y fluxes, the next plane's C, D and z flux (the register queue), C_old, and
// the lane halo (lane 0: C, D of column i-1; lane 31: C, D and the x flux of column i+1).
template <class T>
struct PDRow {
    T qx, cjm, djm, qyl, cjp, djp, qyu, cn, dn, qzn, co, hc, hd, hq;
};

struct PDFlags {
    bool lx, cx, yu, h0, h31c, h31q;
};

template <class T>
__device__ __forceinline__ PDRow<T> pd_load(const PDM<T>& f, int o, bool zu, const PDFlags& fl) {
    PDRow<T> r;
    const int s1 = f.s1, s2 = f.s2;
    r.qx = fl.lx ? __ldg(f.q[0] + o) : T(0);
    r.cjm = r.djm = r.qyl = r.cjp = r.djp = r.qyu = r.cn = r.dn = r.qzn = r.co = T(0);
    r.hc = r.hd = r.hq = T(0);
    if (fl.cx) {
        r.cjm = __ldg(f.C + o - s1);
        r.djm = __ldg(f.D + o - s1);
        r.qyl = __ldg(f.q[1] + o);
        r.qyu = __ldg(f.q[1] + o + s1);
        if (fl.yu) {
            r.cjp = __ldg(f.C + o + s1);
            r.djp = __ldg(f.D + o + s1);
        }
        r.qzn = __ldg(f.q[2] + o + s2);
        if (zu) {
            r.cn = __ldg(f.C + o + s2);
            r.dn = __ldg(f.D + o + s2);
        }
        r.co = __ldg(f.Co + o);
    }
    if (fl.h0) {
        r.hc = __ldg(f.C + o - 1);
        r.hd = __ldg(f.D + o - 1);
    }
    if (fl.h31c) {
        r.hc = __ldg(f.C + o + 1);
        r.hd = __ldg(f.D + o + 1);
    }
    if (fl.h31q) r.hq = __ldg(f.q[0] + o + 1);
    return r;
}

template <class T, int NW, int MINB>
__global__ void __launch_bounds__(32 * NW, MINB)
    ptd_march3d_kernel(const PDM<T> f, int e0, int e1, int e2, int ntx, int nty, int seg_len) {
    using namespace cgk;
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int tx = b % ntx, ty = (b / ntx) % nty, seg = b / (ntx * nty);
    const int ks = seg * seg_len;
    const int i = tx * 32 + lane, j = ty * NW + w;
    if (ks > e2 || j > e1) return;  // whole warp
    const int ke = min(ks + seg_len - 1, e2);
    PDFlags fl;
    fl.cx = i <= e0;      // a cell of the launch range
    fl.lx = i <= e0 + 1;  // column e0+1 passes its stored x flux to the lane below
    fl.yu = j + 1 <= e1;  // the upper y face is computed (else stored)
    fl.h0 = lane == 0 && fl.cx;
    fl.h31c = lane == 31 && i + 1 <= e0;
    fl.h31q = lane == 31 && i + 1 <= e0 + 1;
    const int s2 = f.s2;
    int o = i + j * f.s1 + ks * s2;
    // prologue: C and D of plane ks and the new flux of its lower z face
    T c = T(0), d = T(0), qzl = T(0);
    if (fl.cx) {
        c = __ldg(f.C + o);
        d = __ldg(f.D + o);
        qzl = pd_face(__ldg(f.q[2] + o), __ldg(f.D + o - s2), d, __ldg(f.C + o - s2), c, f.idx[2], f.om);
    }
    PDRow<T> cur = pd_load(f, o, ks + 1 <= e2, fl);
    for (int k = ks; k <= ke; ++k, o += s2) {
        PDRow<T> nxt;
        if (k < ke) nxt = pd_load(f, o + s2, k + 2 <= e2, fl);
        // x faces
        T cl = __shfl_up_sync(FULL, c, 1), dl = __shfl_up_sync(FULL, d, 1);
        if (lane == 0) {
            cl = cur.hc;
            dl = cur.hd;
        }
        const T qxl = fl.cx ? pd_face(cur.qx, dl, d, cl, c, f.idx[0], f.om) : cur.qx;
        T qxu = __shfl_down_sync(FULL, qxl, 1);
        if (lane == 31) qxu = fl.h31c ? pd_face(cur.hq, d, cur.hd, c, cur.hc, f.idx[0], f.om) : cur.hq;
        if (fl.cx) {
            // y and z faces
            const T qyl = pd_face(cur.qyl, cur.djm, d, cur.cjm, c, f.idx[1], f.om);
            const T qyu = fl.yu ? pd_face(cur.qyu, d, cur.djp, c, cur.cjp, f.idx[1], f.om) : cur.qyu;
            const T qzu = k + 1 <= e2 ? pd_face(cur.qzn, d, cur.dn, c, cur.cn, f.idx[2], f.om) : cur.qzn;
            // R = -(C - C_old)/dt - divg(q); C += R dtau_C
            T dv = rmul(rsub(qxu, qxl), f.idx[0]);
            dv = radd(dv, rmul(rsub(qyu, qyl), f.idx[1]));
            dv = radd(dv, rmul(rsub(qzu, qzl), f.idx[2]));
            const T rr = rsub(rmul(-rsub(c, cur.co), f.inv_dt), dv);
            f.Cn[o] = radd(c, rmul(rr, f.dtc));
            f.qn[0][o] = qxl;
            f.qn[1][o] = qyl;
            f.qn[2][o] = qzl;
            qzl = qzu;
        }
        c = cur.cn;
        d = cur.dn;
        cur = nxt;
    }
}

// z planes per segment: the count of segments that fills the SMs' resident blocks in whole
// waves most evenly, with segments of at least 16 planes
inline int pd_seg_len(long tiles, int planes, long resident) {
    int best = planes;
    double best_eff = 0.0;
    for (int ns = 1; ns <= 64; ++ns) {
        const int len = (planes + ns - 1) / ns;
        if (len < 16 && ns > 1) break;
        const double waves = (double)(tiles * ns) / (double)resident;
        const double eff = waves / std::ceil(waves);
        if (eff > best_eff + 1e-3) {
            best_eff = eff;
            best = len;
        }
    }
    return best;
}

template <class T, int NW, int MINB>
cudaError_t launch_pd_ix(const PDM<T>& f, const cg_grid* g, int num_sms, cudaStream_t st) {
    const int e0 = g->n[0] + 1, e1 = g->n[1] + 1, e2 = g->n[2] + 1;
    const int ntx = cg_div_up(e0 + 1, 32), nty = cg_div_up(e1 + 1, NW);
    static const int bps = [] {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ptd_march3d_kernel<T, NW, MINB>, 32 * NW, 0) != cudaSuccess)
            nb = 0;
        return nb > 0 ? nb : 1;
    }();
    const long tiles = (long)ntx * nty;
    const int seg = pd_seg_len(tiles, e2 + 1, (long)num_sms * bps);
    const int nseg = cg_div_up(e2 + 1, seg);
    ptd_march3d_kernel<T, NW, MINB><<<(unsigned)(tiles * nseg), 32 * NW, 0, st>>>(f, e0, e1, e2, ntx, nty, seg);
    return cudaGetLastError();
}

}  // namespace

#include "cg_ptd_tma.cuh"

namespace {

// The tensor maps of one ping-pong direction of a fused run (TMA variants), or none.
struct PdDir {
    const ptdt::Maps* m[kPdHeights] = {};  // per block height (kPdHeight)
    const ptdt::Boxes* b[kPdHeights] = {};
    int* err = nullptr;
};

inline PdDir pd_dir(const PdTma& t, bool ab) {
    PdDir d;
    if (!t.ok) return d;
    for (int h = 0; h < kPdHeights; ++h) {
        d.m[h] = ab ? &t.ab[h] : &t.ba[h];
        d.b[h] = ab ? &t.bab[h] : &t.bba[h];
    }
    d.err = t.err;
    return d;
}

// Shared memory that leaves room for at most `blocks` blocks per SM (228 KB per SM, 1 KB of it
// reserved per block), or what the ring needs when that is more; blocks = 0: the size for the
// widest boxes (max_smem_bytes).
inline int pd_smem_for(int need, int blocks, int widest) {
    if (blocks == 0) return need > widest ? need : widest;
    const int cap = (233472 / blocks - 1024) & ~127;
    return need > cap ? need : cap;
}

// The TMA-fed iteration with blocks of NW rows, a ring of S planes and at most B blocks per SM
// (B = 0: the shared memory of the widest boxes). Measured at 512^3, fewer concurrent blocks
// were faster, and the launch bounds' register budget mattered: the kept layouts are the
// fastest of the sweep.
template <int NW, int MINB, int S, int B>
cudaError_t launch_pd_tma(const PDM<float>& f, const cg_grid* g, int num_sms, cudaStream_t st, const ptdt::Maps& maps,
                          const ptdt::Boxes& bx, int* err) {
    auto kern = ptd_tma_kernel<NW, MINB, S>;
    const int smem = pd_smem_for(ptdt::smem_bytes(S, bx.sf), B, ptdt::max_smem_bytes<NW, S>());
    static const bool attr = [&] {
        const bool r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    (void)attr;
    const int e0 = g->n[0] + 1, e1 = g->n[1] + 1, e2 = g->n[2] + 1;
    const int ntx = cg_div_up(e0 + 1, 32), nty = cg_div_up(e1 + 1, NW);
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 32 * NW, smem) != cudaSuccess || bps < 1) {
        cudaGetLastError();
        bps = 1;
    }
    const long tiles = (long)ntx * nty;
    const int seg = pd_seg_len(tiles, e2 + 1, (long)num_sms * bps);
    const int nseg = cg_div_up(e2 + 1, seg);
    const cg_tma_cfg wc = cg_tma_wait_cfg();
    kern<<<(unsigned)(tiles * nseg), 32 * NW, smem, st>>>(maps, f, bx, e0, e1, e2, ntx, nty, seg, wc.limit_ns, wc.withhold,
                                                         err);
    return cudaGetLastError();
}

// Launch layouts of the fused iteration. Variants 0-3, ptd_march3d_kernel (all without register
// spills for FP32): 8 rows at 4 or 5 blocks per SM, 16 rows at 2, 4 rows at 10; taller blocks
// read fewer y-halo rows, more resident warps keep more loads in flight. Variants 4-7,
// ptd_tma_kernel (inputs staged by TMA; only with tensor maps for the direction), rings of 4
// planes with the shared memory of the widest boxes: blocks of 8, 16, 20 and 24 rows (at 512^3
// 24 rows, 2 blocks per SM, measured fastest; 32 rows, 1 block per SM, 27 % slower).
constexpr int kPdVariants = 8;
constexpr int kPdTmaFirst = 4;

template <class T>
cudaError_t launch_pd_march3d(const PDM<T>& f, const cg_grid* g, int num_sms, cudaStream_t st, int variant,
                              const PdDir& dir = PdDir{}) {
    if constexpr (sizeof(T) == 4) {
        if (variant >= kPdTmaFirst && dir.m[0]) {
            const int h = variant - kPdTmaFirst;
            if (h == 0) return launch_pd_tma<8, 4, 4, 0>(f, g, num_sms, st, *dir.m[0], *dir.b[0], dir.err);
            if (h == 1) return launch_pd_tma<16, 2, 4, 0>(f, g, num_sms, st, *dir.m[1], *dir.b[1], dir.err);
            // launch bounds of one block for 20 and 24 rows: with two, ptxas fits the kernel in
            // 35-36 registers instead of 38, and 24 rows measured 1224 instead of 1050 us at 512^3
            if (h == 2) return launch_pd_tma<20, 1, 4, 0>(f, g, num_sms, st, *dir.m[2], *dir.b[2], dir.err);
            if (h == 3) return launch_pd_tma<24, 1, 4, 0>(f, g, num_sms, st, *dir.m[3], *dir.b[3], dir.err);
        }
    }
    switch (variant) {
        case 1: return launch_pd_ix<T, 8, 5>(f, g, num_sms, st);
        case 2: return launch_pd_ix<T, 16, 2>(f, g, num_sms, st);
        case 3: return launch_pd_ix<T, 4, 10>(f, g, num_sms, st);
        default: return launch_pd_ix<T, 8, 4>(f, g, num_sms, st);
    }
}

// CG_PTD_VARIANT=<0..7> in the environment (read on every call): the fused iteration's layout
// instead of the autotuner's (a TMA variant only where its tensor maps exist).
inline int pd_variant_forced() {
    const char* e = std::getenv("CG_PTD_VARIANT");
    if (!e || !e[0]) return -1;
    const int v = std::atoi(e);
    return v >= 0 && v < kPdVariants ? v : -1;
}

// The fastest layout for this grid and layout, timed on the run's own buffers before its graph
// is captured (the launch writes only the partner buffers) and cached for the process.
template <class T>
int tune_pd(const PDM<T>& f, const cg_grid* g, int num_sms, cudaStream_t st, const PdDir& dir = PdDir{}) {
    const bool tma = dir.m[0] != nullptr;
    const int forced = pd_variant_forced();
    if (forced >= 0) return (forced >= kPdTmaFirst && !tma) ? 0 : forced;
    if (!cg_autotune_enabled()) return 0;
    std::string key = "ptdiff3d";
    for (int d = 0; d < 3; ++d) cg_key_add(key, g->n[d]);
    cg_key_add(key, f.s1);
    cg_key_add(key, f.s2);
    cg_key_add(key, num_sms);
    cg_key_add(key, (int)tma);
    cg_tune_cfg best{0, 0};
    if (cg_tune_lookup(key, &best)) return best.variant;
    float tbest = 1e30f;
    for (int v = 0; v < (tma ? kPdVariants : kPdTmaFirst); ++v) {
        const float t = cgk::time_launches([&] { return launch_pd_march3d<T>(f, g, num_sms, st, v, dir); }, st);
        if (cg_tune_verbose())
            std::fprintf(stderr, "ptdiff3d tune %dx%dx%d: variant %d: %.1f us\n", g->n[0], g->n[1], g->n[2], v,
                         t >= 0.f ? 1e3f * t / 3 : -1.f);
        if (t >= 0.f && t < tbest) {
            tbest = t;
            best = cg_tune_cfg{0, v};
        }
    }
    cudaGetLastError();
    cg_tune_store(key, best);
    return best.variant;
}

template <class T>
PDM<T> make_pdm(const cg_grid* g, const cg_field& C, const cg_field* q, const cg_field& Cn, const cg_field* qn,
                const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    PDM<T> m;
    std::memset(&m, 0, sizeof(m));
    m.C = cg_view<T>(C).p;
    m.Cn = cg_view<T>(Cn).p;
    for (int d = 0; d < 3; ++d) {
        m.q[d] = cg_view<T>(q[d]).p;
        m.qn[d] = cg_view<T>(qn[d]).p;
        m.idx[d] = (T)g->inv_spacing[d];
    }
    m.Co = cg_view<T>(f->C_old).p;
    m.D = cg_view<T>(f->D).p;
    m.s1 = (int)C.stride[1];
    m.s2 = (int)C.stride[2];
    m.om = (T)p->omega_q;
    m.inv_dt = T(1) / (T)p->dt;
    m.dtc = (T)p->dtau_C;
    return m;
}

// cg_ptdiff_run on the fused kernel (3D): partner buffers for C and q in scratch slot 2, with
// the caller's layouts and contents (so the points no iteration writes agree), ping-pong
// between the two sets, and the result copied back after an odd number of iterations.
template <class T>
int run_fused3d(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p, const cg_bc* bc,
                int nsteps, int npt, std::string key) {
    size_t bytes[4], off[4], total = 0;
    const cg_field* src[4] = {&f->C, &f->q[0], &f->q[1], &f->q[2]};
    for (int a = 0; a < 4; ++a) {
        bytes[a] = padded_bytes(*src[a]);
        off[a] = total;
        total += (bytes[a] + 255) & ~(size_t)255;
    }
    int rc = CG_OK;
    char* base = static_cast<char*>(cg_scratch(ctx, 2, total, &rc));
    if (rc) return rc;
    cg_field part[4];
    for (int a = 0; a < 4; ++a) {
        part[a] = *src[a];
        part[a].data = base + off[a];
    }
    const PDM<T> ab = make_pdm<T>(g, f->C, f->q, part[0], part + 1, f, p);
    const PDM<T> ba = make_pdm<T>(g, part[0], part + 1, f->C, f->q, f, p);
    int* err = cg_tma_flag(ctx, &rc);
    if (rc) return rc;
    const PdTma tma = make_pd_tma(f->C, f->q, part[0], part + 1, f->D, f->C_old, err);
    const PdDir dab = pd_dir(tma, true), dba = pd_dir(tma, false);
    const int variant = tune_pd<T>(ab, g, ctx->num_sms, ctx->stream, dab);
    cg_key_add(key, base);
    cg_key_add(key, variant);
    if (variant >= kPdTmaFirst) {
        // the maps encode this call's pointers, and the wait settings are kernel arguments:
        // both are part of the graph's key
        cg_key_add(key, tma.ab[variant - kPdTmaFirst]);
        cg_key_add(key, tma.ba[variant - kPdTmaFirst]);
        cg_key_add(key, cg_tma_wait_cfg());
    }
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int a = 0; a < 4; ++a)
            CG_CUDA(ctx, cudaMemcpyAsync(part[a].data, src[a]->data, bytes[a], cudaMemcpyDeviceToDevice, st));
        for (int s = 0; s < nsteps; ++s) {
            CG_CUDA(ctx, cudaMemcpyAsync(f->C_old.data, f->C.data, bytes[0], cudaMemcpyDeviceToDevice, st));
            for (int it = 0; it < npt; ++it) {
                const cudaError_t le =
                    launch_pd_march3d<T>(it % 2 == 0 ? ab : ba, g, ctx->num_sms, st, variant, it % 2 == 0 ? dab : dba);
                if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "ptdiff fused launch: %s", cudaGetErrorString(le));
                if (bc) {
                    int r = cg_bc_apply_impl(ctx, g, 1, it % 2 == 0 ? &part[0] : &f->C, bc);
                    if (r) return r;
                }
            }
            if (npt % 2)
                for (int a = 0; a < 4; ++a)
                    CG_CUDA(ctx, cudaMemcpyAsync(src[a]->data, part[a].data, bytes[a], cudaMemcpyDeviceToDevice, st));
        }
        return (int)CG_OK;
    });
    if (rc) return rc;
    return variant >= kPdTmaFirst ? cg_tma_check(ctx, err, "ptdiff fused iteration") : CG_OK;
}

// The fused path needs a 3D FP32 grid, no residual output, and one row and plane stride for
// C, C_old, D and the three fluxes (a common pitch and plane height, e.g. Field(...,
// pitch_align, plane_rows)), with every offset in 32 bits.
bool fused3d_ok(const cg_grid* g, const cg_ptdiff_fields* f) {
    if (g->ndim != 3 || f->C.dtype != CG_F32 || cg_present(f->R) || !cg_ptdiff_fused_enabled()) return false;
    const cg_field* all[6] = {&f->C, &f->C_old, &f->D, &f->q[0], &f->q[1], &f->q[2]};
    for (const cg_field* a : all)
        for (int d = 1; d < 3; ++d)
            if (a->stride[d] != f->C.stride[d]) return false;
    const long last = (long)(g->n[0] + 3) + (long)(g->n[1] + 3) * f->C.stride[1] + (long)(g->n[2] + 3) * f->C.stride[2];
    return last < 2147483647L;
}

}  // namespace

extern "C" int cg_ptdiff_update_q(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                                  const cg_ptdiff_params* p) {
    int rc = check_ptdiff(ctx, grid, f, p);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    return PDISPATCH(launch_q, f->C.dtype, grid->ndim, ctx, grid, f, p);
}

extern "C" int cg_ptdiff_update_C(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                                  const cg_ptdiff_params* p) {
    int rc = check_ptdiff(ctx, grid, f, p);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    return PDISPATCH(launch_C, f->C.dtype, grid->ndim, ctx, grid, f, p);
}

extern "C" int cg_ptdiff_run(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p,
                             const cg_bc* bc, int nsteps, int npt) {
    int rc = check_ptdiff(ctx, grid, f, p);
    if (rc) return rc;
    if (nsteps < 0 || npt < 0) return cg_fail(ctx, CG_ERR_ARG, "ptdiff_run: negative counts");
    if (f->C.stride[1] != f->C_old.stride[1] || f->C.stride[2] != f->C_old.stride[2])
        return cg_fail(ctx, CG_ERR_ARG, "ptdiff_run: C and C_old must share a layout");
    if (nsteps == 0 || npt == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    std::string key = "ptdiff_run";
    cg_key_add(key, *grid);
    cg_key_add(key, *f);
    cg_key_add(key, *p);
    cg_bc none;
    std::memset(&none, 0, sizeof(none));
    cg_key_add(key, bc ? *bc : none);
    cg_key_add(key, nsteps);
    cg_key_add(key, npt);
    if (fused3d_ok(grid, f)) return run_fused3d<float>(ctx, grid, f, p, bc, nsteps, npt, key + "fused3d");
    const size_t cbytes = padded_bytes(f->C);
    const int dtype = f->C.dtype, nd = grid->ndim;
    dim3 bq, bcl;
    if ((rc = PDISPATCH(ptdiff_blocks, dtype, nd, ctx, grid, f, p, &bq, &bcl))) return rc;
    cg_key_add(key, bq);
    cg_key_add(key, bcl);
    return cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int s = 0; s < nsteps; ++s) {
            // update_old: C_old <- C (whole padded array)
            CG_CUDA(ctx, cudaMemcpyAsync(f->C_old.data, f->C.data, cbytes, cudaMemcpyDeviceToDevice, st));
            for (int it = 0; it < npt; ++it) {
                int r = PDISPATCH(launch_q, dtype, nd, ctx, grid, f, p, bq);
                if (r) return r;
                r = PDISPATCH(launch_C, dtype, nd, ctx, grid, f, p, bcl);
                if (r) return r;
                if (bc && (r = cg_bc_apply_impl(ctx, grid, 1, &f->C, bc))) return r;
            }
        }
        return (int)CG_OK;
    });
}

// ---- adjoint: gradient with respect to the diffusivity ------------------------------------
//
// One implicit step is C' = S C with S = (I - dt L_D)^-1 and L_D C = divg(lerp(D) d C). With
// the boundary rules folded in, I - dt L_D is symmetric on the interior cells, so the adjoint
// of a step is the same step: lambda^n = S lambda^{n+1} (a PT step with C_old = lambda^{n+1} and
// zero boundary values). For a misfit J(C^N), perturbing D gives
//   dJ = sum_n dt lambda^n . (dL_D C^{n+1}),
// and, collecting the terms of each face f between cells l and r = l + e_d (the face's D is the
// mean of its two cells, so each cell carries half of it),
//   dJ/dD_c = dt sum_n sum_{faces f of c} 1/2 (C_r - C_l) idx_d^2 (lambda_l [l interior]
//                                                                  - lambda_r [r interior]).
// This kernel adds `scale` times one step's term (scale = dt) for lambda = lambda^n and
// C = C^{n+1} at every interior cell (logical indices 1..n).
namespace {

template <class T, int ND>
__global__ void ptdiff_grad_kernel(const DF<T> lam, const DF<T> C, const DF<T> grad, T scale, T idx0, T idx1,
                                   T idx2, int n0, int n1, int n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y + 1 : 0;
    const int k = ND > 2 ? blockIdx.z + 1 : 0;
    if (i > n0 || (ND > 1 && j > n1) || (ND > 2 && k > n2)) return;
    const int c[3] = {i, j, k}, n[3] = {n0, n1, n2};
    const T idx[3] = {idx0, idx1, idx2};
    T s = T(0);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        for (int side = 0; side < 2; ++side) {
            int l[3] = {c[0], c[1], c[2]}, r[3] = {c[0], c[1], c[2]};
            if (side == 0) l[d] -= 1;  // lower face: (c - e_d, c)
            else r[d] += 1;            // upper face: (c, c + e_d)
            const T dC = (C(r[0], r[1], r[2]) - C(l[0], l[1], l[2])) * idx[d];
            const T ll = l[d] >= 1 ? lam(l[0], l[1], l[2]) : T(0);
            const T lr = r[d] <= n[d] ? lam(r[0], r[1], r[2]) : T(0);
            s += T(0.5) * dC * (ll - lr) * idx[d];
        }
    }
    grad(i, j, k) = grad(i, j, k) + scale * s;
}

}  // namespace

extern "C" int cg_ptdiff_gradient_D(cg_ctx* ctx, const cg_grid* grid, const cg_field* lam, const cg_field* C,
                                    double scale, const cg_field* grad) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "ptdiff_gradient_D: ctx is NULL");
    if (!grid || !lam || !C || !grad) return cg_fail(ctx, CG_ERR_ARG, "ptdiff_gradient_D: NULL argument");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    const int dtype = grad->dtype, nd = grid->ndim;
    if ((rc = cg_check_field(ctx, grid, *grad, dtype, 0, "grad"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *lam, dtype, 0, "lambda"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *C, dtype, 0, "C"))) return rc;
    cudaSetDevice(ctx->device);
    const int n0 = grid->n[0], n1 = nd > 1 ? grid->n[1] : 1, n2 = nd > 2 ? grid->n[2] : 1;
    const dim3 block(nd == 1 ? 256 : 32, nd == 1 ? 1 : 8);
    const dim3 gr(cg_div_up(n0, block.x), nd > 1 ? cg_div_up(n1, block.y) : 1, nd > 2 ? n2 : 1);
    auto go = [&](auto tag) {
        using T = decltype(tag);
        const DF<T> l = cg_view<T>(*lam), c = cg_view<T>(*C), g = cg_view<T>(*grad);
        const T i0 = (T)grid->inv_spacing[0], i1 = (T)grid->inv_spacing[1], i2 = (T)grid->inv_spacing[2];
        if (nd == 1) ptdiff_grad_kernel<T, 1><<<gr, block, 0, ctx->stream>>>(l, c, g, (T)scale, i0, i1, i2, n0, n1, n2);
        else if (nd == 2) ptdiff_grad_kernel<T, 2><<<gr, block, 0, ctx->stream>>>(l, c, g, (T)scale, i0, i1, i2, n0, n1, n2);
        else ptdiff_grad_kernel<T, 3><<<gr, block, 0, ctx->stream>>>(l, c, g, (T)scale, i0, i1, i2, n0, n1, n2);
    };
    if (dtype == CG_F64) go(double(0));
    else go(float(0));
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// ---- one implicit step solved to a tolerance -----------------------------------------------
//
// The step's equation at every interior cell (logical 1..n) is
//   R(C) = -(C - C_old)/dt - divg(q(C)) = 0,   q_d = -lerp(D -> face_d) ∂_d C
// (the converged state of the PT iterations; the ghost planes follow from bc!). Its measure
// is err = max|R| dt over the interior. The PT iterations' own residual uses the damped PT
// flux instead of q(C). Two forms:
// - FP64: the PT iterations of cg_ptdiff_run on the caller's fields, checked every ncheck
//   iterations.
// - FP32 defect correction: with the FP64 defect R of C, the correction d solves the same
//   linear step with C_old' = dt R and the boundary rules' homogeneous form
//   (d/dt - divg(lerp(D) ∇d) = R). FP32 PT iterations of the fused kernel solve it, from zero,
//   on FP32 work arrays that share one layout. The inner loop stops at
//   max(eps/2, inner_rtol err), or when it stops improving. Then C += d, bc!(C) follows, and
//   the FP64 defect again. Only the defect and the update run in FP64.
namespace {

// exact-flux residual at interior cells of C (FP64), its max |R| dt, and optionally
// C_old' = dt R into an FP32 array of the pool
template <class T, class TO>
__global__ void pd_residual_kernel(const DF<T> C, const DF<T> Co, const DF<T> D, T idx0, T idx1, T idx2, T inv_dt,
                                   T dt, int n0, int n1, int n2, const DF<TO> out, int has_out,
                                   unsigned long long* slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const bool in = i <= n0 && j <= n1 && k <= n2;
    T r = T(0);
    if (in) {
        const T c = C(i, j, k), dc = D(i, j, k);
        const T idx[3] = {idx0, idx1, idx2};
        T dv = T(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int di = d == 0, dj = d == 1, dk = d == 2;
            const T cl = C(i - di, j - dj, k - dk), cr = C(i + di, j + dj, k + dk);
            const T dl = D(i - di, j - dj, k - dk), dr = D(i + di, j + dj, k + dk);
            const T ql = -fma(T(0.5), dc - dl, dl) * ((c - cl) * idx[d]);
            const T qr = -fma(T(0.5), dr - dc, dc) * ((cr - c) * idx[d]);
            dv += (qr - ql) * idx[d];
        }
        r = -(c - Co(i, j, k)) * inv_dt - dv;
        if (has_out) out(i, j, k) = (TO)(r * dt);
    }
    cgk::block_max_bits(in ? cgk::bits_of(fabs(r * dt)) : 0ull, slot);
}

// C += d at interior cells (FP64 += FP32)
__global__ void pd_update_kernel(const DF<double> C, const DF<float> d, int n0, int n1, int n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > n0 || j > n1 || k > n2) return;
    C(i, j, k) = C(i, j, k) + (double)d(i, j, k);
}

// FP64 -> FP32 over the padded extent of D (every point the fused kernel reads)
__global__ void pd_to32_kernel(const DF<double> a, const DF<float> b, int n0, int n1, int n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > n0 + 2 || j > n1 + 2 || k > n2 + 2) return;
    b(i, j, k) = (float)a(i, j, k);
}

// q = -lerp(D) ∂C on the faces of the launch range [0, n+1]^3 (the converged flux)
__global__ void pd_flux_kernel(const DF<double> C, const DF<double> D, DF<double> q0, DF<double> q1, DF<double> q2,
                               double idx0, double idx1, double idx2, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i > e0 || j > e1) return;
    const double c = C(i, j, k), dc = D(i, j, k);
    const DF<double> q[3] = {q0, q1, q2};
    const double idx[3] = {idx0, idx1, idx2};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int di = d == 0, dj = d == 1, dk = d == 2;
        const double dl = D(i - di, j - dj, k - dk);
        q[d](i, j, k) = -fma(0.5, dc - dl, dl) * ((c - C(i - di, j - dj, k - dk)) * idx[d]);
    }
}

double decode_max(unsigned long long v, bool* bad) {
    double x;
    std::memcpy(&x, &v, 8);
    if (v >= 0x7FF0000000000000ull) *bad = true;
    return x;
}

// max|R| dt of C (FP64 fields); writes C_old' = dt R into `out` when given
template <class TO>
int residual64(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p, const cg_field* out,
               double* err, bool* bad) {
    CG_CUDA(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    const dim3 block(32, 8), grid(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8), g->n[2]);
    const double inv_dt = 1.0 / p->dt;
    pd_residual_kernel<double, TO><<<grid, block, 0, ctx->stream>>>(
        cg_view<double>(f->C), cg_view<double>(f->C_old), cg_view<double>(f->D), g->inv_spacing[0], g->inv_spacing[1],
        g->inv_spacing[2], inv_dt, p->dt, g->n[0], g->n[1], g->n[2], out ? cg_view<TO>(*out) : DF<TO>{}, out != nullptr,
        ctx->d_red);
    CG_CHECK_LAUNCH(ctx);
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *err = decode_max(ctx->h_red[0], bad);
    return CG_OK;
}

// max|r| dt of the correction's equation (FP32 pool arrays: d, C_old' = dt R, D)
int residual32(cg_ctx* ctx, const cg_grid* g, const cg_field& d, const cg_field& co, const cg_field& D,
               const cg_ptdiff_params* p, double* err, bool* bad) {
    CG_CUDA(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    const dim3 block(32, 8), grid(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8), g->n[2]);
    pd_residual_kernel<float, float><<<grid, block, 0, ctx->stream>>>(
        cg_view<float>(d), cg_view<float>(co), cg_view<float>(D), (float)g->inv_spacing[0], (float)g->inv_spacing[1],
        (float)g->inv_spacing[2], 1.0f / (float)p->dt, (float)p->dt, g->n[0], g->n[1], g->n[2], DF<float>{}, 0, ctx->d_red);
    CG_CHECK_LAUNCH(ctx);
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned u = (unsigned)ctx->h_red[0];
    float x;
    std::memcpy(&x, &u, 4);
    if (u >= 0x7F800000u) *bad = true;
    *err = (double)x;
    return CG_OK;
}

// FP32 array of the pool: n[] of location loc, one row pitch and plane height for all
cg_field pool_field(char* base, size_t off, const cg_grid* g, int loc_mask, long pitch, long rows) {
    cg_field a;
    std::memset(&a, 0, sizeof(a));
    a.data = base + off;
    a.dtype = CG_F32;
    a.ndim = 3;
    for (int d = 0; d < 3; ++d) {
        const bool v = (loc_mask >> d) & 1;
        a.n[d] = g->n[d] + (v ? 1 : 0);
        a.loc[d] = v ? CG_VERTEX : CG_CENTER;
        a.halo[d] = 1;
    }
    a.stride[0] = 1;
    a.stride[1] = pitch;
    a.stride[2] = pitch * rows;
    return a;
}

int solve_fp64(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p, const cg_bc* bc,
               const cg_solve_opts* o, cg_solve_result* res) {
    const int ncheck = std::max(1, o->ncheck);
    std::string key = "ptdiff_chunk64";
    cg_key_add(key, *g);
    cg_key_add(key, *f);
    cg_key_add(key, *p);
    cg_key_add(key, *bc);
    cg_key_add(key, ncheck);
    int it = 0;
    for (;;) {
        double err = 0;
        bool bad = false;
        int rc = residual64<double>(ctx, g, f, p, nullptr, &err, &bad);
        if (rc) return rc;
        res->checks++;
        res->err[0] = err;
        if (bad) return cg_fail(ctx, CG_ERR_NONFINITE, "ptdiff_solve (FP64): non-finite residual");
        if (err < o->eps) {
            res->converged = 1;
            break;
        }
        if (it >= o->max_iter) break;
        rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
            (void)st;
            for (int k = 0; k < ncheck; ++k) {
                int r = launch_q<double, 3>(ctx, g, f, p);
                if (r) return r;
                if ((r = launch_C<double, 3>(ctx, g, f, p))) return r;
                if ((r = cg_bc_apply_impl(ctx, g, 1, &f->C, bc))) return r;
            }
            return (int)CG_OK;
        });
        if (rc) return rc;
        it += ncheck;
    }
    res->iterations = it;
    return CG_OK;
}

int solve_dc(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p, const cg_bc* bc,
             const cg_solve_opts* o, cg_solve_result* res) {
    // FP32 pool: d, d', q x3, q' x3, C_old' (dt R), D; logical x index 0 of every row on a
    // 128-byte boundary (31 elements of front), so that a warp's 32 columns store whole lines.
    // Measured at 512^3 with a bc! launch per iteration: the TMA-fed iteration takes 1128 us
    // per iteration in this layout and 1221 us with the first padded element aligned, where
    // the register-fed kernel's best is 1195 us.
    const long front = 31, pitch = ((front + g->n[0] + 5 + 31) / 32) * 32, rows = g->n[1] + 5;
    const size_t per = (size_t)pitch * rows * (g->n[2] + 5) * sizeof(float);
    const size_t per_al = (per + 255) & ~(size_t)255;
    int rc = CG_OK;
    char* base = static_cast<char*>(cg_scratch(ctx, 4, per_al * 10 + 256, &rc));
    if (rc) return rc;
    // an array's data pointer sits `front` elements past the pool's 256-byte boundaries
    base += front * sizeof(float);
    const int qm[3] = {1, 2, 4};
    cg_field dA = pool_field(base, 0, g, 0, pitch, rows), dB = pool_field(base, per_al, g, 0, pitch, rows);
    cg_field qA[3], qB[3];
    for (int d = 0; d < 3; ++d) {
        qA[d] = pool_field(base, per_al * (2 + d), g, qm[d], pitch, rows);
        qB[d] = pool_field(base, per_al * (5 + d), g, qm[d], pitch, rows);
    }
    cg_field co = pool_field(base, per_al * 8, g, 0, pitch, rows), D32 = pool_field(base, per_al * 9, g, 0, pitch, rows);
    cg_ptdiff_fields w;
    std::memset(&w, 0, sizeof(w));
    w.C = dA;
    w.C_old = co;
    w.D = D32;
    for (int d = 0; d < 3; ++d) w.q[d] = qA[d];
    {
        const dim3 block(32, 8), grid(cg_div_up(g->n[0] + 4, 32), cg_div_up(g->n[1] + 4, 8), g->n[2] + 4);
        pd_to32_kernel<<<grid, block, 0, ctx->stream>>>(cg_view<double>(f->D), cg_view<float>(D32), g->n[0], g->n[1],
                                                         g->n[2]);
        CG_CHECK_LAUNCH(ctx);
    }
    // the correction's boundary rules: the caller's kinds with zero values
    cg_bc bc0 = *bc;
    for (int d = 0; d < 3; ++d) {
        bc0.value[d][0] = bc0.value[d][1] = 0.0;
        bc0.values[d][0] = bc0.values[d][1] = nullptr;
    }
    const PDM<float> ab = make_pdm<float>(g, dA, qA, dB, qB, &w, p);
    const PDM<float> ba = make_pdm<float>(g, dB, qB, dA, qA, &w, p);
    int* perr = cg_tma_flag(ctx, &rc);
    if (rc) return rc;
    const PdTma tma = make_pd_tma(dA, qA, dB, qB, D32, co, perr);
    const PdDir dab = pd_dir(tma, true), dba = pd_dir(tma, false);
    const int variant = tune_pd<float>(ab, g, ctx->num_sms, ctx->stream, dab);
    const int nchunk = std::max(2, o->ncheck + (o->ncheck & 1));
    std::string key = "ptdiff_dc_chunk";
    cg_key_add(key, *g);
    cg_key_add(key, base);
    cg_key_add(key, *p);
    cg_key_add(key, bc0);
    cg_key_add(key, nchunk);
    cg_key_add(key, variant);
    cg_key_add(key, cg_tma_wait_cfg());
    const dim3 ib(32, 8), ig(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8), g->n[2]);
    int total = 0;
    const size_t zero_bytes = per_al * 8;  // d, d', q, q' (the first eight arrays)
    for (int outer = 0;; ++outer) {
        double err = 0;
        bool bad = false;
        CG_CUDA(ctx, cudaMemsetAsync(co.data, 0, per, ctx->stream));
        if ((rc = residual64<float>(ctx, g, f, p, &co, &err, &bad))) return rc;
        res->checks++;
        res->err[0] = err;
        if (bad) return cg_fail(ctx, CG_ERR_NONFINITE, "ptdiff_solve (FP32): non-finite FP64 residual");
        if (err < o->eps) {
            res->converged = 1;
            break;
        }
        if (outer >= o->max_outer || total >= o->max_iter) break;
        // FP32 correction from zero
        CG_CUDA(ctx, cudaMemsetAsync(base, 0, zero_bytes, ctx->stream));
        const double target = std::max(0.5 * o->eps, o->inner_rtol * err);
        // the FP32 floor of the correction's measure sits near eps_32 D dt / h^2 of the outer
        // error: a loop that gains nothing over max(4 ncheck, n) iterations has reached it
        const int nmax = std::max(g->n[0], std::max(g->n[1], g->n[2]));
        const int window = std::max(4 * nchunk, nmax);
        double best = 1e300;
        int since = 0;
        while (total < o->max_iter) {
            rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
                for (int it = 0; it < nchunk; ++it) {
                    const cudaError_t le = launch_pd_march3d<float>(it % 2 == 0 ? ab : ba, g, ctx->num_sms, st, variant,
                                                                    it % 2 == 0 ? dab : dba);
                    if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "ptdiff fused launch: %s", cudaGetErrorString(le));
                    int r = cg_bc_apply_impl(ctx, g, 1, it % 2 == 0 ? &dB : &dA, &bc0);
                    if (r) return r;
                }
                return (int)CG_OK;
            });
            if (rc) return rc;
            total += nchunk;
            double e32 = 0;
            bool bad32 = false;
            if ((rc = residual32(ctx, g, dA, co, D32, p, &e32, &bad32))) return rc;
            res->checks++;
            if (bad32) return cg_fail(ctx, CG_ERR_NONFINITE, "ptdiff_solve (FP32): non-finite correction residual");
            if (e32 < target) break;
            if (e32 < 0.9 * best) {
                best = e32;
                since = 0;
            } else if ((since += nchunk) >= window) {
                break;  // the FP32 floor: back to the FP64 defect
            }
        }
        if (variant >= kPdTmaFirst && (rc = cg_tma_check(ctx, perr, "ptdiff fused iteration"))) return rc;
        pd_update_kernel<<<ig, ib, 0, ctx->stream>>>(cg_view<double>(f->C), cg_view<float>(dA), g->n[0], g->n[1], g->n[2]);
        CG_CHECK_LAUNCH(ctx);
        if ((rc = cg_bc_apply_impl(ctx, g, 1, &f->C, bc))) return rc;
        res->outer++;
    }
    // the converged flux into q
    {
        const dim3 block(32, 8), grid(cg_div_up(g->n[0] + 2, 32), cg_div_up(g->n[1] + 2, 8), g->n[2] + 2);
        pd_flux_kernel<<<grid, block, 0, ctx->stream>>>(cg_view<double>(f->C), cg_view<double>(f->D),
                                                         cg_view<double>(f->q[0]), cg_view<double>(f->q[1]),
                                                         cg_view<double>(f->q[2]), g->inv_spacing[0], g->inv_spacing[1],
                                                         g->inv_spacing[2], g->n[0] + 1, g->n[1] + 1);
        CG_CHECK_LAUNCH(ctx);
    }
    res->iterations = total;
    return CG_OK;
}

}  // namespace

extern "C" int cg_ptdiff_solve(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p,
                               const cg_bc* bc, const cg_solve_opts* o, cg_solve_result* res) {
    int rc = check_ptdiff(ctx, grid, f, p);
    if (rc) return rc;
    if (!bc || !o || !res) return cg_fail(ctx, CG_ERR_ARG, "ptdiff_solve: NULL bc, opts or result");
    if (grid->ndim != 3) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "ptdiff_solve: 3D grids only");
    if (f->C.dtype != CG_F64) return cg_fail(ctx, CG_ERR_ARG, "ptdiff_solve: FP64 fields (the FP32 form is internal)");
    for (int d = 0; d < 3; ++d)
        for (int s = 0; s < 2; ++s)
            if (bc->kind[d][s] != CG_BC_DIRICHLET && bc->kind[d][s] != CG_BC_NEUMANN)
                return cg_fail(ctx, CG_ERR_UNSUPPORTED,
                               "ptdiff_solve: every side needs a Dirichlet or Neumann rule (the residual is over the interior)");
    if (o->precision != CG_F64 && o->precision != CG_F32)
        return cg_fail(ctx, CG_ERR_ARG, "ptdiff_solve: precision must be CG_F64 or CG_F32");
    if (o->max_iter < 0 || !(o->eps > 0)) return cg_fail(ctx, CG_ERR_ARG, "ptdiff_solve: bad max_iter or eps");
    const long last = (long)(grid->n[0] + 5 + 63) * (grid->n[1] + 5) * (grid->n[2] + 5);
    if (o->precision == CG_F32 && last >= 2147483647L)
        return cg_fail(ctx, CG_ERR_UNSUPPORTED, "ptdiff_solve: grid too large for 32-bit offsets in the FP32 form");
    cudaSetDevice(ctx->device);
    std::memset(res, 0, sizeof(*res));
    CG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    rc = o->precision == CG_F64 ? solve_fp64(ctx, grid, f, p, bc, o, res) : solve_dc(ctx, grid, f, p, bc, o, res);
    if (rc) return rc;
    CG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    CG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->seconds = ms * 1e-3;
    if (!res->converged)
        return cg_fail(ctx, CG_ERR_NOCONV, "ptdiff_solve: not converged (err %.3e) after %d iterations", res->err[0],
                       res->iterations);
    return CG_OK;
}
