// cg_sia_ensemble.cu — an ensemble of independent shallow-ice solves of uneven grid sizes
// (examples/sia.jl:7-16,71-81 per member) advanced together. Every phase of a time step covers
// the tiles of all members (a per-member tile prefix table maps tiles to members), and the
// adaptive Δt of every member is computed on the device. The `nsteps` loop is one launch per
// phase, replayed from a CUDA graph. With CG_SIA_PERSISTENT=1 (and cooperative launch support)
// it is instead ONE persistent cooperative launch with grid barriers between the phases. Both
// forms give the same bits. The graph is the default: on GB300 the tiles are bound by the FP64
// pipe, so residency saves nothing, and a grid barrier costs more than a kernel boundary in a
// replayed graph (64 members of 128^2..1024^2: 2.49 vs 2.41 ms per step; of 32^2..128^2:
// 70 vs 62 us).
//
// Boundary conditions are folded into the kernels with the values of the reference's bc!:
// q.x => (x = Dirichlet()) writes 0 on the boundary faces i = 1, n+1 (q.y likewise), and
// H => Neumann() copies the first interior value into the ghost layer, corners taking the
// value of the diagonal interior cell (the x rule runs last and reads the y ghost).
//
// The step is bound by the FP64 pipe, so FP64 work is traded for memory traffic:
// - S = B + H is kept per cell in a scratch array. The H kernel updates it with the new
//   thickness, including the ghost layer; the cells beyond it never change.
// - The D kernel hands its lower-face surface gradients to the q kernel through the q arrays.
// Every value is the one the direct form computes, with the same operations in the same order.
#include <vector>

#include "cg_common.cuh"
#include "cg_sia_kernels.cuh"

void* cg_scratch(cg_ctx* ctx, int slot, size_t bytes, int* rc);

namespace {

template <class T>
struct Member {
    DF<T> H, B, qx, qy, D, S;
    T Gamma, As, beta, ela, m_max, idx, idy;
    T Gn2, Asn;  // Gamma (n+2) and As n, for the taped derivatives of D
    double dx2, cfl, dt_max;
    int n, nx, ny;
    int tiles_D, tiles_I;  // tiles of the [0, n] and [1, n] ranges (32 x blockDim.y each)
    // taped runs: the member's tape block within a step's block (cgsia layout: 256 bytes of
    // words, then kArrays arrays of `tab` bytes in H's layout, H's origin at element `orig`)
    long long toff, tab, orig;
};

// The member's tape array k (cgsia::TapeArray) of the step whose block starts at `sb`.
template <class T>
__device__ __forceinline__ DF<T> tape_arr(const Member<T>& v, char* sb, int k) {
    DF<T> a = v.H;
    a.p = reinterpret_cast<T*>(sb + v.toff + 256 + (long long)k * v.tab) + v.orig;
    return a;
}
template <class T>
__device__ __forceinline__ DF<unsigned char> tape_flags(const Member<T>& v, char* sb) {
    DF<unsigned char> a;
    a.p = reinterpret_cast<unsigned char*>(sb + v.toff + 256 + (long long)cgsia::kFL * v.tab) + v.orig;
    a.s1 = v.H.s1;
    a.s2 = v.H.s2;
    return a;
}
template <class T>
__device__ __forceinline__ cgsia::TapeWords* tape_words(const Member<T>& v, char* sb) {
    return reinterpret_cast<cgsia::TapeWords*>(sb + v.toff);
}

struct Words {
    unsigned long long dmax;
    double dt;
    double t;
    double pad;
};

using cgsia::bits_of;

// The block's member descriptor, copied once into shared memory (every thread of the block
// calls it before reading the member).
// The leading barrier lets a block that loops over tiles (the persistent kernel) call it once
// per tile: the previous tile's reads of the descriptor and of the block-max scratch are done.
template <class T>
__device__ __forceinline__ const Member<T>& member_of(const Member<T>* mem, int m) {
    __shared__ __align__(16) unsigned long long words[(sizeof(Member<T>) + 7) / 8];
    __syncthreads();
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(mem + m);
    for (int k = tid; k < (int)((sizeof(Member<T>) + 7) / 8); k += blockDim.x * blockDim.y) words[k] = src[k];
    __syncthreads();
    return *reinterpret_cast<const Member<T>*>(words);
}

// block -> (member, tile) through the inclusive prefix of per-member tile counts
__device__ __forceinline__ int find_member(const int* prefix, int nm, int blk) {
    int lo = 0, hi = nm - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] > blk) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

template <class T, bool TAPE = false>
__device__ __forceinline__ void ens_D_tile(const Member<T>* mem, const int* prefix, int nm, Words* w, int blk,
                                           char* sb = nullptr) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 1 + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x;
    const int j = (t / tx) * (int)blockDim.y + threadIdx.y;
    const bool in = i <= v.nx && j <= v.ny;
    T d = T(0);
    if (in) {
        // ∇S at the cell's faces, interpolated to the cell; vmag and D (examples/sia.jl:43-49)
        const T s = v.S(i, j, 0);
        const T a0 = (s - v.S(i - 1, j, 0)) * v.idx;
        const T a1 = (v.S(i + 1, j, 0) - s) * v.idx;
        const T b0 = (s - v.S(i, j - 1, 0)) * v.idy;
        const T b1 = (v.S(i, j + 1, 0) - s) * v.idy;
        const T ax = fma(T(0.5), a1 - a0, a0);
        const T ay = fma(T(0.5), b1 - b0, b0);
        const T h = v.H(i, j, 0);
        T dh, ex, ey, gf;
        if (TAPE)
            d = cgsia::D_and_factors(h, ax, ay, v.Gamma, v.As, v.Gn2, v.Asn, v.n, &dh, &ex, &ey, &gf);
        else
            d = cgsia::D_cell(h, ax, ay, v.Gamma, v.As, v.n);
        v.D(i, j, 0) = d;
        if (i >= 1 && j >= 1) {  // the lower faces' gradients, for the q kernel
            v.qx(i, j, 0) = a0;
            v.qy(i, j, 0) = b0;
            if (TAPE) {
                using namespace cgsia;
                tape_arr(v, sb, kD)(i, j, 0) = d;
                tape_arr(v, sb, kGX)(i, j, 0) = a0;
                tape_arr(v, sb, kGY)(i, j, 0) = b0;
                tape_arr(v, sb, kDH)(i, j, 0) = dh;
                tape_arr(v, sb, kEX)(i, j, 0) = ex;
                tape_arr(v, sb, kEY)(i, j, 0) = ey;
                tape_arr(v, sb, kGF)(i, j, 0) = gf;
            }
        }
    }
    cgsia::block_max_bits(in && i >= 1 && j >= 1 ? bits_of(d) : 0ull, &w[m].dmax);
}

// S = B + H over [-1, n+1]^2 (the D kernel's stencil), once per run
template <class T>
__device__ __forceinline__ void ens_S_tile(const Member<T>* mem, const int* prefix, int nm, int blk) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 3 + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x - 1;
    const int j = (t / tx) * (int)blockDim.y + threadIdx.y - 1;
    if (i > v.nx + 1 || j > v.ny + 1) return;
    v.S(i, j, 0) = v.B(i, j, 0) + v.H(i, j, 0);
}

template <class T>
__device__ __forceinline__ void ens_q_tile(const Member<T>* mem, const int* prefix, int nm, int blk) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x + 1;
    const int j = (t / tx) * (int)blockDim.y + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    const T dc = v.D(i, j, 0), dl = v.D(i - 1, j, 0), dd = v.D(i, j - 1, 0);
    const T Dx = fma(T(0.5), dc - dl, dl);
    const T Dy = fma(T(0.5), dc - dd, dd);
    // q = -lerp(D) ∂S with ∂S left in q by the D kernel; bc!(q.x => (x = Dirichlet())): the
    // boundary faces i = 1 and n+1 are 0 (q.y likewise)
    v.qx(i, j, 0) = i == 1 ? T(0) : -Dx * v.qx(i, j, 0);
    v.qy(i, j, 0) = j == 1 ? T(0) : -Dy * v.qy(i, j, 0);
    if (i == v.nx) v.qx(i + 1, j, 0) = T(0);
    if (j == v.ny) v.qy(i, j + 1, 0) = T(0);
}

template <class T, bool TAPE = false>
__device__ __forceinline__ void ens_dt_member(const Member<T>* mem, Words* w, int m, char* sb = nullptr) {
    const Member<T>& v = mem[m];
    const unsigned long long b = w[m].dmax;
    const double dmax = sizeof(T) == 8 ? __longlong_as_double((long long)b) : (double)__int_as_float((int)(unsigned)b);
    const T q = (T)v.dx2 / (T)dmax / (T)v.cfl;
    double d = fmin((double)q, v.dt_max);
    bool capped = !((double)q < v.dt_max);
    if (!(dmax > 0.0)) {
        d = v.dt_max;
        capped = true;
    }
    w[m].dt = d;
    w[m].t = w[m].t + d;
    w[m].dmax = 0ull;
    if (TAPE) {
        cgsia::TapeWords* tw = tape_words(v, sb);
        tw->dmax = b;
        tw->arg = ~0ull;
        tw->dt = d;
        tw->capped = capped ? 1.0 : 0.0;
    }
}

template <class T, bool TAPE = false>
__device__ __forceinline__ void ens_H_tile(const Member<T>* mem, const int* prefix, int nm, const Words* w, int blk,
                                           char* sb = nullptr) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x + 1;
    const int j = (t / tx) * (int)blockDim.y + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    const T dt = (T)w[m].dt;
    const T h = v.H(i, j, 0);
    // M = min(beta (S - ela), m_max) and H = max(H + dt (-divg q + M), 0), as std::min/max
    // (a NaN propagates as in the reference)
    const T x = v.beta * (v.S(i, j, 0) - v.ela);
    const T mb = v.m_max < x ? v.m_max : x;
    T dv = (v.qx(i + 1, j, 0) - v.qx(i, j, 0)) * v.idx;
    dv = dv + (v.qy(i, j + 1, 0) - v.qy(i, j, 0)) * v.idy;
    const T W = -dv + mb;
    const T u = h + dt * W;
    const T hn = u < T(0.0) ? T(0.0) : u;
    if (TAPE) {
        using namespace cgsia;
        tape_arr(v, sb, kW)(i, j, 0) = W;
        tape_flags(v, sb)(i, j, 0) = (unsigned char)((u > T(0) ? 1 : 0) + (v.m_max < x ? 0 : 2));
        cgsia::TapeWords* tw = tape_words(v, sb);
        if (bits_of(v.D(i, j, 0)) == tw->dmax) atomicMin(&tw->arg, (unsigned long long)((long)j * (v.nx + 2) + i));
    }
    v.H(i, j, 0) = hn;
    v.S(i, j, 0) = v.B(i, j, 0) + hn;
    // bc!(H => Neumann()): ghost layer and corners from the first interior cells
    const bool l = i == 1, r = i == v.nx, b = j == 1, tp = j == v.ny;
    auto ghost = [&](int gi, int gj) {
        v.H(gi, gj, 0) = hn;
        v.S(gi, gj, 0) = v.B(gi, gj, 0) + hn;
    };
    if (l) ghost(0, j);
    if (r) ghost(v.nx + 1, j);
    if (b) ghost(i, 0);
    if (tp) ghost(i, v.ny + 1);
    if (l && b) ghost(0, 0);
    if (r && b) ghost(v.nx + 1, 0);
    if (l && tp) ghost(0, v.ny + 1);
    if (r && tp) ghost(v.nx + 1, v.ny + 1);
}

template <class T, bool TAPE = false>
__global__ void ens_D_kernel(const Member<T>* mem, const int* prefix, int nm, Words* w, char* sb) {
    ens_D_tile<T, TAPE>(mem, prefix, nm, w, blockIdx.x, sb);
}
template <class T>
__global__ void ens_S_kernel(const Member<T>* mem, const int* prefix, int nm) {
    ens_S_tile(mem, prefix, nm, blockIdx.x);
}
template <class T>
__global__ void ens_q_kernel(const Member<T>* mem, const int* prefix, int nm) {
    ens_q_tile(mem, prefix, nm, blockIdx.x);
}
template <class T, bool TAPE = false>
__global__ void ens_dt_kernel(const Member<T>* mem, int nm, Words* w, char* sb) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nm) ens_dt_member<T, TAPE>(mem, w, m, sb);
}
template <class T, bool TAPE = false>
__global__ void ens_H_kernel(const Member<T>* mem, const int* prefix, int nm, const Words* w, char* sb) {
    ens_H_tile<T, TAPE>(mem, prefix, nm, w, blockIdx.x, sb);
}

// ---- one persistent launch for the whole run ------------------------------------------------
//
// The same tiles and arithmetic as the per-phase kernels: the resident blocks of a cooperative
// launch loop over each phase's tiles, with a grid barrier between the phases. Per step:
// D and the block maxima; barrier; Δt of every member (block 0) and the fluxes; barrier; the
// thickness; barrier. The barrier counts arrivals on one monotonic word. Its waits give up
// after a time limit (two seconds of the GPU's global timer unless the host sets another) and
// set a timeout flag: the kernel then returns, and the host reports the error. A cooperative
// launch keeps every block resident, so the waits end.
struct GridBar {
    unsigned long long arrived;  // arrivals since the launch: barrier k completes at (k + 1) x expect
    int timeout;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier `k` (0, 1, ...) of the launch: one relaxed add per block, then a wait of at most
// `limit_ns` until `expect` blocks (the grid's size) have added. Nothing is reset, so the last
// block to arrive has no extra work.
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned expect, unsigned long long limit_ns,
                                             unsigned long long& k) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const unsigned long long target = (++k) * expect;
        __threadfence();
        atomicAdd(&b->arrived, 1ull);
        volatile unsigned long long* va = &b->arrived;
        const unsigned long long t0 = globaltimer_ns();
        while (*va < target) {
            if (globaltimer_ns() - t0 > limit_ns) {
                atomicExch(&b->timeout, 1);
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&b->timeout == 0;
}

template <class T>
__global__ void __launch_bounds__(256, 8) ens_persistent_kernel(const Member<T>* mem, const int* pD, const int* pI,
                                                             const int* pS, int nm, int totD, int totI, int totS,
                                                             Words* w, int nsteps, GridBar* bar, unsigned expect,
                                                             unsigned long long limit_ns) {
    const unsigned nb = gridDim.x;
    unsigned long long k = 0;
    for (int b = blockIdx.x; b < totS; b += nb) ens_S_tile(mem, pS, nm, b);
    if (!grid_barrier(bar, expect, limit_ns, k)) return;
    for (int s = 0; s < nsteps; ++s) {
        for (int b = blockIdx.x; b < totD; b += nb) ens_D_tile(mem, pD, nm, w, b);
        if (!grid_barrier(bar, expect, limit_ns, k)) return;
        if (blockIdx.x == 0)
            for (int m = threadIdx.x + blockDim.x * threadIdx.y; m < nm; m += blockDim.x * blockDim.y)
                ens_dt_member(mem, w, m);
        for (int b = blockIdx.x; b < totI; b += nb) ens_q_tile(mem, pI, nm, b);
        if (!grid_barrier(bar, expect, limit_ns, k)) return;
        for (int b = blockIdx.x; b < totI; b += nb) ens_H_tile(mem, pI, nm, w, b);
        if (!grid_barrier(bar, expect, limit_ns, k)) return;
    }
}

// ---- tape of a taped ensemble run ------------------------------------------------------------
//
// A 256-byte header, then per step one block holding every member's tape in turn, each in the
// single-member layout of cgsia (words, then kArrays arrays in the member's H layout).
struct EnsTape {
    std::vector<long long> toff, tab, orig;
    size_t step_bytes = 0;
};

inline EnsTape ens_tape_layout(int nm, const cg_sia_member* ms, size_t elem) {
    EnsTape e;
    e.toff.resize(nm);
    e.tab.resize(nm);
    e.orig.resize(nm);
    size_t off = 0;
    for (int m = 0; m < nm; ++m) {
        const cgsia::TapeGeom g = cgsia::tape_geom(ms[m].H, elem);
        e.toff[m] = (long long)off;
        e.tab[m] = (long long)g.abytes;
        e.orig[m] = (long long)cg_origin_offset(ms[m].H);
        off += g.step_bytes;
    }
    e.step_bytes = off;
    return e;
}

struct EnsTapeHeader {
    unsigned long long magic;
    int dtype, nm, nsteps, pad;
    unsigned long long step_bytes, hash;
};
constexpr unsigned long long kEnsTapeMagic = 0x31534e4541544953ull;  // "SIATENS1"

// FNV-1a over the members' layouts, grid spacings and parameters: a reverse sweep checks it
// against its own
inline unsigned long long ens_tape_hash(int nm, const cg_sia_member* ms, const cg_sia_params* ps) {
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        for (size_t k = 0; k < n; ++k) h = (h ^ c[k]) * 1099511628211ull;
    };
    for (int m = 0; m < nm; ++m) {
        const cg_field& H = ms[m].H;
        const long long lay[8] = {ms[m].grid.n[0], ms[m].grid.n[1], H.n[0], H.n[1], H.halo[0], H.halo[1],
                                  (long long)H.stride[0], (long long)H.stride[1]};
        mix(lay, sizeof(lay));
        const double pr[9] = {ps[m].Gamma,  ps[m].As,     ps[m].beta,
                              ps[m].ela,    ps[m].m_max,  ps[m].cfl,
                              ps[m].dt_max, ms[m].grid.inv_spacing[0], ms[m].grid.inv_spacing[1]};
        mix(pr, sizeof(pr));
        mix(&ps[m].n, sizeof(int));
    }
    return h;
}

template <class T>
int run_t(cg_ctx* ctx, int nm, const cg_sia_member* ms, const cg_sia_params* ps, int nsteps, double* t_host,
          char* tape = nullptr) {
    // scratch slot 3: [members][prefix D][prefix I][words][D arrays...]
    size_t off = 0;
    const size_t mem_off = off;
    off += ((size_t)nm * sizeof(Member<T>) + 255) & ~(size_t)255;
    const size_t pD_off = off;
    off += ((size_t)nm * sizeof(int) + 255) & ~(size_t)255;
    const size_t pI_off = off;
    off += ((size_t)nm * sizeof(int) + 255) & ~(size_t)255;
    const size_t pS_off = off;
    off += ((size_t)nm * sizeof(int) + 255) & ~(size_t)255;
    const size_t w_off = off;
    off += ((size_t)nm * sizeof(Words) + 255) & ~(size_t)255;
    const size_t bar_off = off;
    off += 256;
    std::vector<size_t> d_off(nm), s_off(nm);
    for (int m = 0; m < nm; ++m) {
        const cg_field& H = ms[m].H;
        const size_t cnt = (size_t)H.stride[1] * (H.n[1] + 4 * H.halo[1]);
        d_off[m] = off;
        off += (cnt * sizeof(T) + 255) & ~(size_t)255;
        s_off[m] = off;
        off += (cnt * sizeof(T) + 255) & ~(size_t)255;
    }
    int rc = CG_OK;
    char* base = static_cast<char*>(cg_scratch(ctx, 3, off, &rc));
    if (rc) return rc;
    std::vector<Member<T>> hm(nm);
    std::vector<int> pD(nm), pI(nm), pS(nm);
    const EnsTape et = ens_tape_layout(nm, ms, sizeof(T));
    int totD = 0, totI = 0, totS = 0;
    Member<T>* dmem = reinterpret_cast<Member<T>*>(base + mem_off);
    int* dpD = reinterpret_cast<int*>(base + pD_off);
    int* dpI = reinterpret_cast<int*>(base + pI_off);
    int* dpS = reinterpret_cast<int*>(base + pS_off);
    Words* dw = reinterpret_cast<Words*>(base + w_off);
    // members and tile prefix tables for tiles of 32 x ty points, uploaded to the scratch
    auto layout = [&](int ty) -> int {
        totD = totI = totS = 0;
        for (int m = 0; m < nm; ++m) {
            const cg_sia_member& s = ms[m];
            const cg_sia_params& p = ps[m];
            Member<T>& v = hm[m];
            std::memset(&v, 0, sizeof(v));
            v.H = cg_view<T>(s.H);
            v.B = cg_view<T>(s.B);
            v.qx = cg_view<T>(s.q[0]);
            v.qy = cg_view<T>(s.q[1]);
            v.D = v.H;
            v.D.p = reinterpret_cast<T*>(base + d_off[m]) + cg_origin_offset(s.H);
            v.S = v.H;
            v.S.p = reinterpret_cast<T*>(base + s_off[m]) + cg_origin_offset(s.H);
            v.Gamma = (T)p.Gamma;
            v.As = (T)p.As;
            v.beta = (T)p.beta;
            v.ela = (T)p.ela;
            v.m_max = (T)p.m_max;
            v.Gn2 = v.Gamma * T(p.n + 2);
            v.Asn = v.As * T(p.n);
            v.idx = (T)s.grid.inv_spacing[0];
            v.idy = (T)s.grid.inv_spacing[1];
            const double dx = std::min(s.grid.spacing[0], s.grid.spacing[1]);
            v.dx2 = (double)((T)dx * (T)dx);
            v.cfl = p.cfl;
            v.dt_max = p.dt_max;
            v.n = p.n;
            v.nx = s.grid.n[0];
            v.ny = s.grid.n[1];
            v.tiles_D = cg_div_up(v.nx + 1, 32) * cg_div_up(v.ny + 1, ty);
            v.tiles_I = cg_div_up(v.nx, 32) * cg_div_up(v.ny, ty);
            if (tape) {
                v.toff = et.toff[m];
                v.tab = et.tab[m];
                v.orig = et.orig[m];
            }
            totD += v.tiles_D;
            totI += v.tiles_I;
            totS += cg_div_up(v.nx + 3, 32) * cg_div_up(v.ny + 3, ty);
            pD[m] = totD;
            pI[m] = totI;
            pS[m] = totS;
        }
        CG_CUDA(ctx, cudaMemcpyAsync(dmem, hm.data(), nm * sizeof(Member<T>), cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(dpD, pD.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(dpI, pI.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(dpS, pS.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemsetAsync(dw, 0, nm * sizeof(Words), ctx->stream));
        // the host tables are read by the copies above before the next layout call rewrites them
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return CG_OK;
    };
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess) coop = 0;
    const bool persistent = coop && !tape && cg_sia_persistent_enabled();
    // tile height: 8 rows for the persistent kernel, else the forced or autotuned choice
    int ty = 8;
    if (!persistent) {
        const int forced = cg_sia_tile_rows_forced();
        if (forced) {
            ty = forced;
        } else if (cg_autotune_enabled()) {
            std::string tkey = "sia_ensemble_tiles";
            cg_key_add(tkey, (int)sizeof(T));
            cg_key_add(tkey, ctx->num_sms);
            for (int m = 0; m < nm; ++m) {
                cg_key_add(tkey, ms[m].grid.n[0]);
                cg_key_add(tkey, ms[m].grid.n[1]);
            }
            cg_tune_cfg tc{0, 0};
            if (cg_tune_lookup(tkey, &tc)) {
                ty = tc.variant;
            } else {
                // time the D and flux phases of one step for each tile height; neither changes
                // the thickness (D, the face gradients, the fluxes and S = B + H are recomputed
                // by the run, and the words are cleared by the next layout call)
                float best = 1e30f;
                for (int cand : {4, 8, 16}) {
                    if ((rc = layout(cand))) return rc;
                    const dim3 bk(32, cand);
                    const float t = cgk::time_launches(
                        [&] {
                            ens_S_kernel<T><<<totS, bk, 0, ctx->stream>>>(dmem, dpS, nm);
                            ens_D_kernel<T><<<totD, bk, 0, ctx->stream>>>(dmem, dpD, nm, dw, nullptr);
                            ens_q_kernel<T><<<totI, bk, 0, ctx->stream>>>(dmem, dpI, nm);
                            return cudaGetLastError();
                        },
                        ctx->stream);
                    if (cg_tune_verbose())
                        std::fprintf(stderr, "sia ensemble tune (%d members): 32x%d tiles: %.1f us\n", nm, cand,
                                     t >= 0.f ? 1e3f * t / 3 : -1.f);
                    if (t >= 0.f && t < best) {
                        best = t;
                        ty = cand;
                    }
                }
                cudaGetLastError();
                cg_tune_store(tkey, cg_tune_cfg{0, ty});
            }
        }
    }
    if ((rc = layout(ty))) return rc;
    const dim3 block(32, ty);
    // cooperative-launch support and residency of the persistent kernel are queried per call on
    // this context's device (a process may hold contexts on different GPU models)
    if (persistent) {
        // the whole run in one cooperative launch of the resident blocks
        int bps = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ens_persistent_kernel<T>, 256, 0) != cudaSuccess) bps = 0;
        if (bps < 1) return cg_fail(ctx, CG_ERR_CUDA, "sia_ensemble_run: the persistent kernel does not fit on an SM");
        GridBar* bar = reinterpret_cast<GridBar*>(base + bar_off);
        CG_CUDA(ctx, cudaMemsetAsync(bar, 0, sizeof(GridBar), ctx->stream));
        const Member<T>* cmem = dmem;
        const int *cpD = dpD, *cpI = dpI, *cpS = dpS;
        int anm = nm, atD = totD, atI = totI, atS = totS, ans = nsteps;
        const unsigned nblocks = (unsigned)(bps * ctx->num_sms);
        const cg_barrier_cfg bcfg = cg_sia_barrier_cfg();
        unsigned expect = nblocks + (unsigned)bcfg.withheld;
        unsigned long long limit_ns = bcfg.limit_ns;
        void* args[] = {&cmem, &cpD, &cpI, &cpS, &anm, &atD, &atI, &atS, &dw, &ans, &bar, &expect, &limit_ns};
        CG_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)ens_persistent_kernel<T>, dim3(nblocks), block,
                                                 args, 0, ctx->stream));
        int timed_out = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&timed_out, &bar->timeout, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (timed_out) return cg_fail(ctx, CG_ERR_TIMEOUT, "sia_ensemble_run: a grid barrier of the persistent kernel timed out");
    } else {
    std::string key = "sia_ensemble";
    cg_key_add(key, ty);
    cg_key_add(key, nm);
    cg_key_add(key, nsteps);
    cg_key_add(key, base);
    cg_key_add(key, tape);
    key.append(reinterpret_cast<const char*>(hm.data()), nm * sizeof(Member<T>));
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        ens_S_kernel<T><<<totS, block, 0, st>>>(dmem, dpS, nm);
        for (int s = 0; s < nsteps; ++s) {
            if (tape) {
                char* sb = tape + 256 + (size_t)s * et.step_bytes;
                ens_D_kernel<T, true><<<totD, block, 0, st>>>(dmem, dpD, nm, dw, sb);
                ens_q_kernel<T><<<totI, block, 0, st>>>(dmem, dpI, nm);
                ens_dt_kernel<T, true><<<cg_div_up(nm, 64), 64, 0, st>>>(dmem, nm, dw, sb);
                ens_H_kernel<T, true><<<totI, block, 0, st>>>(dmem, dpI, nm, dw, sb);
            } else {
                ens_D_kernel<T><<<totD, block, 0, st>>>(dmem, dpD, nm, dw, nullptr);
                ens_q_kernel<T><<<totI, block, 0, st>>>(dmem, dpI, nm);
                ens_dt_kernel<T><<<cg_div_up(nm, 64), 64, 0, st>>>(dmem, nm, dw, nullptr);
                ens_H_kernel<T><<<totI, block, 0, st>>>(dmem, dpI, nm, dw, nullptr);
            }
            CG_CHECK_LAUNCH(ctx);
        }
        return (int)CG_OK;
    });
    if (rc) return rc;
    }
    if (t_host) {
        std::vector<Words> hw(nm);
        CG_CUDA(ctx, cudaMemcpyAsync(hw.data(), dw, nm * sizeof(Words), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int m = 0; m < nm; ++m) t_host[m] = hw[m].t;
    }
    return CG_OK;
}

// ---- reverse sweep over an ensemble tape ----------------------------------------------------
//
// The reverse step of cg_sia_adjoint_run applied to every member at once: per step, the cell
// kernel over all members' interior tiles, one block per member for the ordered sums of its
// tiles' partials and the dt term at its argmax cell, and the gather kernel over all tiles.
template <class T>
struct AdjMember {
    DF<T> L, Wk, lo, pax, pay;  // lambda and work (in/out by turns), the step's scratch
    DF<double> aG, aE;          // per-cell sums over the sweep's steps of dJ/dGamma and dJ/dela
    T beta, idx, idy;
    int nx, ny;
    long long toff, tab, orig;
};

template <class T>
__device__ __forceinline__ const AdjMember<T>& adj_member_of(const AdjMember<T>* am, int m) {
    __shared__ __align__(16) unsigned long long words[(sizeof(AdjMember<T>) + 7) / 8];
    __syncthreads();
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(am + m);
    for (int k = tid; k < (int)((sizeof(AdjMember<T>) + 7) / 8); k += blockDim.x * blockDim.y) words[k] = src[k];
    __syncthreads();
    return *reinterpret_cast<const AdjMember<T>*>(words);
}

template <class T>
__device__ __forceinline__ DF<T> adj_tape(const AdjMember<T>& v, const char* sb, int k) {
    DF<T> a = v.L;
    a.p = reinterpret_cast<T*>(const_cast<char*>(sb) + v.toff + 256 + (long long)k * v.tab) + v.orig;
    return a;
}

template <class T>
__device__ __forceinline__ DF<unsigned char> adj_flags(const AdjMember<T>& v, const char* sb) {
    DF<unsigned char> a;
    a.p = reinterpret_cast<unsigned char*>(const_cast<char*>(sb) + v.toff + 256 + (long long)cgsia::kFL * v.tab) + v.orig;
    a.s1 = v.L.s1;
    a.s2 = v.L.s2;
    return a;
}

template <class T>
__device__ __forceinline__ T ens_mu(const DF<unsigned char>& fl, const DF<T>& lam, int i, int j) {
    return (fl(i, j, 0) & 1) ? lam(i, j, 0) : T(0);
}

// Cell tiles of the reverse step: 31 owned columns x 8 rows. Every face term is computed once
// and used by both its cells: lane l computes the lower x face of its cell and lane l - 1 takes
// it as its upper face (shuffle); row r computes its lower y face and row r - 1 takes it
// through shared memory (the top row computes the face above it). Lane 31 only supplies the
// face of lane 30. Each cell sums its face terms in the order lower x, upper x, lower y,
// upper y, as a cell that evaluates all four itself does.
constexpr int kCW = 31;

template <class T>
__global__ void __launch_bounds__(256) ens_adj_cell_kernel(const AdjMember<T>* am, const int* prefix, int nm,
                                                           const char* sb, int parity, double* part) {
    using namespace cgsia;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ T fdy[8][32], fsy[8][32];
    const int blk = blockIdx.x;
    const int m = find_member(prefix, nm, blk);
    const AdjMember<T>& v = adj_member_of(am, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + kCW - 1) / kCW;
    const int lane = threadIdx.x, row = threadIdx.y;
    const int i = (t % tx) * kCW + lane + 1;
    const int j = (t / tx) * 8 + row + 1;
    const bool in = i <= v.nx && j <= v.ny;
    const bool own = in && lane < kCW;
    const DF<T> lam = parity ? v.Wk : v.L;
    const DF<unsigned char> FL = adj_flags(v, sb);
    const DF<T> D = adj_tape(v, sb, kD);
    const TapeWords* w = reinterpret_cast<const TapeWords*>(sb + v.toff);
    const T dt = (T)w->dt;
    const T dtx = dt * v.idx, dty = dt * v.idy;
    T muc = T(0), dc = T(0);
    if (in) {
        muc = ens_mu(FL, lam, i, j);
        dc = D(i, j, 0);
    }
    // the lower x face (face i, cells i-1 and i) and the lower y face (face j)
    T tDx = T(0), tSx = T(0), tDy = T(0), tSy = T(0);
    if (in && i >= 2) {
        const T px = dtx * (muc - ens_mu(FL, lam, i - 1, j));
        const T dl = D(i - 1, j, 0);
        tDx = -T(0.5) * px * adj_tape(v, sb, kGX)(i, j, 0);
        tSx = fma(T(0.5), dc - dl, dl) * px * v.idx;
    }
    if (in && j >= 2) {
        const T py = dty * (muc - ens_mu(FL, lam, i, j - 1));
        const T dl = D(i, j - 1, 0);
        tDy = -T(0.5) * py * adj_tape(v, sb, kGY)(i, j, 0);
        tSy = fma(T(0.5), dc - dl, dl) * py * v.idy;
    }
    fdy[row][lane] = tDy;
    fsy[row][lane] = tSy;
    T tDu = T(0), tSu = T(0);
    if (row == 7 && in && j + 1 <= v.ny) {  // the face above the tile
        const T py = dty * (ens_mu(FL, lam, i, j + 1) - muc);
        const T dr = D(i, j + 1, 0);
        tDu = -T(0.5) * py * adj_tape(v, sb, kGY)(i, j + 1, 0);
        tSu = fma(T(0.5), dr - dc, dc) * py * v.idy;
    }
    const T tDr = __shfl_down_sync(FULL, tDx, 1), tSr = __shfl_down_sync(FULL, tSx, 1);
    __syncthreads();
    if (row < 7) {
        tDu = fdy[row + 1][lane];
        tSu = fsy[row + 1][lane];
    }
    double sdt = 0.0;
    if (own) {
        T pD = T(0), pS = T(0);
        if (i >= 2) {
            pD += tDx;
            pS += -tSx;
        }
        if (i + 1 <= v.nx) {
            pD += tDr;
            pS += tSr;
        }
        if (j >= 2) {
            pD += tDy;
            pS += -tSy;
        }
        if (j + 1 <= v.ny) {
            pD += tDu;
            pS += tSu;
        }
        // the mass balance's direct terms: d H'/d H = 1 + dt beta and d H'/d ela = -dt beta
        // where it is not capped (the step's constants, once per thread)
        const bool mM = (FL(i, j, 0) & 2) != 0;
        const T dtb = dt * v.beta;
        const T lo = mM ? muc * (T(1) + dtb) : muc;
        v.lo(i, j, 0) = lo + pD * adj_tape(v, sb, kDH)(i, j, 0) + pS;
        v.pax(i, j, 0) = pD * adj_tape(v, sb, kEX)(i, j, 0);
        v.pay(i, j, 0) = pD * adj_tape(v, sb, kEY)(i, j, 0);
        sdt = (double)(muc * adj_tape(v, sb, kW)(i, j, 0));
        v.aG(i, j, 0) += (double)(pD * adj_tape(v, sb, kGF)(i, j, 0));
        if (mM) v.aE(i, j, 0) -= (double)(muc * dtb);
    }
    const double a = block_sum(sdt);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[blk] = a;
}

// Block m (1024 threads): dJ/ddt of member m's step, its tiles' partials summed in a fixed
// order; then the dt term at its argmax cell (when dt was not capped) into lo, pax, pay and
// the per-cell dJ/dGamma sum there.
template <class T>
__global__ void __launch_bounds__(1024) ens_adj_sum_kernel(const AdjMember<T>* am, const int* prefix, const char* sb,
                                                           const double* part) {
    using namespace cgsia;
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ double red[32];
    const int m = blockIdx.x;
    const int b0 = m ? prefix[m - 1] : 0, b1 = prefix[m];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double x = 0.0;
    for (int b = b0 + tid; b < b1; b += blockDim.x) x += part[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    if (lane == 0) red[warp] = x;
    __syncthreads();
    if (warp != 0) return;
    x = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    if (lane != 0) return;
    const AdjMember<T>& v = am[m];
    const TapeWords* w = reinterpret_cast<const TapeWords*>(sb + v.toff);
    if (w->capped == 0.0 && w->arg != ~0ull) {
        const unsigned long long bb = w->dmax;
        const double dmax = sizeof(T) == 8 ? __longlong_as_double((long long)bb) : (double)__int_as_float((int)(unsigned)bb);
        const T pD = (T)(-x * w->dt / dmax);
        const int i = (int)(w->arg % (unsigned long long)(v.nx + 2));
        const int j = (int)(w->arg / (unsigned long long)(v.nx + 2));
        v.lo(i, j, 0) = v.lo(i, j, 0) + pD * adj_tape(v, sb, kDH)(i, j, 0);
        v.pax(i, j, 0) = v.pax(i, j, 0) + pD * adj_tape(v, sb, kEX)(i, j, 0);
        v.pay(i, j, 0) = v.pay(i, j, 0) + pD * adj_tape(v, sb, kEY)(i, j, 0);
        v.aG(i, j, 0) += (double)(pD * adj_tape(v, sb, kGF)(i, j, 0));
    }
}

// End of the sweep: per 32 x 8 tile, the sums of the per-cell dJ/dGamma and dJ/dela arrays,
// then (one block per member) their ordered sums into acc[2m], acc[2m + 1].
template <class T>
__global__ void __launch_bounds__(256) ens_adj_tile_sums_kernel(const AdjMember<T>* am, const int* prefix, int nm,
                                                                double* part, int ntot) {
    const int blk = blockIdx.x;
    const int m = find_member(prefix, nm, blk);
    const AdjMember<T>& v = adj_member_of(am, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x + 1;
    const int j = (t / tx) * 8 + threadIdx.y + 1;
    const bool in = i <= v.nx && j <= v.ny;
    const double g = cgsia::block_sum(in ? v.aG(i, j, 0) : 0.0);
    const double e = cgsia::block_sum(in ? v.aE(i, j, 0) : 0.0);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        part[blk] = g;
        part[ntot + blk] = e;
    }
}

__global__ void __launch_bounds__(1024) ens_adj_final_kernel(const int* prefix, const double* part, int ntot, double* acc) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ double red[2][32];
    const int m = blockIdx.x;
    const int b0 = m ? prefix[m - 1] : 0, b1 = prefix[m];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double x[2] = {0.0, 0.0};
    for (int b = b0 + tid; b < b1; b += blockDim.x)
        for (int k = 0; k < 2; ++k) x[k] += part[(size_t)k * ntot + b];
    for (int k = 0; k < 2; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[k] += __shfl_xor_sync(FULL, x[k], o);
        if (lane == 0) red[k][warp] = x[k];
    }
    __syncthreads();
    if (warp != 0) return;
    for (int k = 0; k < 2; ++k) {
        double y = lane < (int)(blockDim.x >> 5) ? red[k][lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(FULL, y, o);
        if (lane == 0) acc[2 * m + k] = y;
    }
}

// lambda_n of every member from lo and the neighbours' pax, pay (the ghost cells' terms folded
// into the interior cells they copy); parity 0 writes Wk, 1 writes L. copy: L = Wk instead.
template <class T>
__global__ void __launch_bounds__(256) ens_adj_out_kernel(const AdjMember<T>* am, const int* prefix, int nm, int parity,
                                                          int copy) {
    const int blk = blockIdx.x;
    const int m = find_member(prefix, nm, blk);
    const AdjMember<T>& v = adj_member_of(am, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x + 1;
    const int j = (t / tx) * 8 + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    if (copy) {
        v.L(i, j, 0) = v.Wk(i, j, 0);
        return;
    }
    const T hx = T(0.5) * v.idx, hy = T(0.5) * v.idy;
    auto PX = [&](int a, int b) { return (a >= 1 && a <= v.nx) ? v.pax(a, b, 0) : T(0); };
    auto PY = [&](int a, int b) { return (b >= 1 && b <= v.ny) ? v.pay(a, b, 0) : T(0); };
    T r = v.lo(i, j, 0) + hx * (PX(i - 1, j) - PX(i + 1, j)) + hy * (PY(i, j - 1) - PY(i, j + 1));
    if (i == 1) r += -hx * v.pax(1, j, 0);
    if (i == v.nx) r += hx * v.pax(v.nx, j, 0);
    if (j == 1) r += -hy * v.pay(i, 1, 0);
    if (j == v.ny) r += hy * v.pay(i, v.ny, 0);
    (parity ? v.L : v.Wk)(i, j, 0) = r;
}

template <class T>
int adjoint_run_t(cg_ctx* ctx, int nm, const cg_sia_member* ms, const cg_sia_params* ps, int N, const char* tape,
                  const cg_field* lam, const cg_field* work, double* dJ) {
    const EnsTape et = ens_tape_layout(nm, ms, sizeof(T));
    std::vector<int> pI(nm), pC(nm);
    std::vector<size_t> aoff(nm);
    int totI = 0, totC = 0;
    // scratch slot 7: [members][prefix][partials 3 x tiles][acc 2 x members][lo, pax, pay per member]
    size_t off = 0;
    const size_t mem_off = off;
    off += ((size_t)nm * sizeof(AdjMember<T>) + 255) & ~(size_t)255;
    const size_t p_off = off;
    off += ((size_t)nm * sizeof(int) + 255) & ~(size_t)255;
    const size_t pc_off = off;
    off += ((size_t)nm * sizeof(int) + 255) & ~(size_t)255;
    for (int m = 0; m < nm; ++m) {
        totI += cg_div_up(ms[m].grid.n[0], 32) * cg_div_up(ms[m].grid.n[1], 8);
        totC += cg_div_up(ms[m].grid.n[0], kCW) * cg_div_up(ms[m].grid.n[1], 8);
        pI[m] = totI;
        pC[m] = totC;
    }
    const size_t part_off = off;
    off += ((size_t)std::max(totC, 2 * totI) * sizeof(double) + 255) & ~(size_t)255;
    const size_t acc_off = off;
    off += ((size_t)2 * nm * sizeof(double) + 255) & ~(size_t)255;
    for (int m = 0; m < nm; ++m) {
        aoff[m] = off;
        off += 3 * (size_t)et.tab[m];
    }
    // the per-cell FP64 sums of every member, in one region (zeroed once per sweep)
    std::vector<size_t> doff(nm);
    const size_t sums_off = off;
    for (int m = 0; m < nm; ++m) {
        doff[m] = off;
        off += 2 * cgsia::tape_geom(ms[m].H, sizeof(double)).abytes;
    }
    const size_t sums_bytes = off - sums_off;
    int rc = CG_OK;
    char* base = static_cast<char*>(cg_scratch(ctx, 7, off, &rc));
    if (rc) return rc;
    std::vector<AdjMember<T>> hm(nm);
    for (int m = 0; m < nm; ++m) {
        AdjMember<T>& v = hm[m];
        std::memset(&v, 0, sizeof(v));
        v.L = cg_view<T>(lam[m]);
        v.Wk = cg_view<T>(work[m]);
        DF<T>* sc[3] = {&v.lo, &v.pax, &v.pay};
        for (int a = 0; a < 3; ++a) {
            *sc[a] = v.L;
            sc[a]->p = reinterpret_cast<T*>(base + aoff[m] + (size_t)a * et.tab[m]) + cg_origin_offset(lam[m]);
        }
        const size_t dab = cgsia::tape_geom(ms[m].H, sizeof(double)).abytes;
        DF<double>* sd[2] = {&v.aG, &v.aE};
        for (int a = 0; a < 2; ++a) {
            sd[a]->p = reinterpret_cast<double*>(base + doff[m] + (size_t)a * dab) + cg_origin_offset(lam[m]);
            sd[a]->s1 = v.L.s1;
            sd[a]->s2 = v.L.s2;
        }
        v.beta = (T)ps[m].beta;
        v.idx = (T)ms[m].grid.inv_spacing[0];
        v.idy = (T)ms[m].grid.inv_spacing[1];
        v.nx = ms[m].grid.n[0];
        v.ny = ms[m].grid.n[1];
        v.toff = et.toff[m];
        v.tab = et.tab[m];
        v.orig = et.orig[m];
    }
    AdjMember<T>* dmem = reinterpret_cast<AdjMember<T>*>(base + mem_off);
    int* dp = reinterpret_cast<int*>(base + p_off);
    int* dpc = reinterpret_cast<int*>(base + pc_off);
    double* part = reinterpret_cast<double*>(base + part_off);
    double* acc = reinterpret_cast<double*>(base + acc_off);
    CG_CUDA(ctx, cudaMemcpyAsync(dmem, hm.data(), nm * sizeof(AdjMember<T>), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dp, pI.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dpc, pC.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    std::string key = "sia_ensemble_adjoint";
    cg_key_add(key, nm);
    cg_key_add(key, N);
    cg_key_add(key, base);
    cg_key_add(key, tape);
    key.append(reinterpret_cast<const char*>(hm.data()), nm * sizeof(AdjMember<T>));
    const dim3 block(32, 8);
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        CG_CUDA(ctx, cudaMemsetAsync(base + sums_off, 0, sums_bytes, st));
        for (int r = 0; r < N; ++r) {
            const char* sb = tape + 256 + (size_t)(N - 1 - r) * et.step_bytes;
            ens_adj_cell_kernel<T><<<totC, block, 0, st>>>(dmem, dpc, nm, sb, r & 1, part);
            ens_adj_sum_kernel<T><<<nm, 1024, 0, st>>>(dmem, dpc, sb, part);
            ens_adj_out_kernel<T><<<totI, block, 0, st>>>(dmem, dp, nm, r & 1, 0);
            CG_CHECK_LAUNCH(ctx);
        }
        if (N & 1) ens_adj_out_kernel<T><<<totI, block, 0, st>>>(dmem, dp, nm, 0, 1);
        ens_adj_tile_sums_kernel<T><<<totI, block, 0, st>>>(dmem, dp, nm, part, totI);
        ens_adj_final_kernel<<<nm, 1024, 0, st>>>(dp, part, totI, acc);
        CG_CHECK_LAUNCH(ctx);
        return (int)CG_OK;
    });
    if (rc) return rc;
    std::vector<double> h(2 * (size_t)nm);
    CG_CUDA(ctx, cudaMemcpyAsync(h.data(), acc, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (dJ)
        for (size_t k = 0; k < h.size(); ++k) dJ[k] += h[k];
    return CG_OK;
}

int check_ensemble(cg_ctx* ctx, int nmembers, const cg_sia_member* members, const cg_sia_params* params,
                   const char* who) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "%s: ctx is NULL", who);
    if (nmembers < 1 || !members || !params) return cg_fail(ctx, CG_ERR_ARG, "%s: no members", who);
    const int dtype = members[0].H.dtype;
    for (int m = 0; m < nmembers; ++m) {
        const cg_sia_member& s = members[m];
        int rc = cg_check_grid(ctx, &s.grid);
        if (rc) return rc;
        if (s.grid.ndim != 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "%s: member %d is not 2D", who, m);
        if ((rc = cg_check_field(ctx, &s.grid, s.H, dtype, 0, "H"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.B, dtype, 0, "B"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.q[0], dtype, 1, "q.x"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.q[1], dtype, 2, "q.y"))) return rc;
        if (params[m].n < 1 || params[m].n > 16 || params[m].cfl <= 0 || params[m].dt_max <= 0)
            return cg_fail(ctx, CG_ERR_ARG, "%s: bad parameters for member %d", who, m);
    }
    return CG_OK;
}

}  // namespace

// The reverse sweep over `nsteps` taped steps whose blocks start at tape + 256, every member in
// each launch; cg_sia_adjoint_run calls it with one member (a single-member tape has the same
// step blocks). Only the members' grids and H layouts are read.
int cg_sia_reverse_impl(cg_ctx* ctx, int nm, const cg_sia_member* ms, const cg_sia_params* ps, int nsteps,
                        const char* tape, const cg_field* lam, const cg_field* work, double* dJ) {
    return ms[0].H.dtype == CG_F64 ? adjoint_run_t<double>(ctx, nm, ms, ps, nsteps, tape, lam, work, dJ)
                                   : adjoint_run_t<float>(ctx, nm, ms, ps, nsteps, tape, lam, work, dJ);
}

extern "C" int cg_sia_ensemble_run(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                   const cg_sia_params* params, int nsteps, double* t_host) {
    int rc = check_ensemble(ctx, nmembers, members, params, "sia_ensemble_run");
    if (rc) return rc;
    if (nsteps < 0) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run: nsteps < 0");
    cudaSetDevice(ctx->device);
    if (nsteps == 0) {
        if (t_host)
            for (int m = 0; m < nmembers; ++m) t_host[m] = 0.0;
        return CG_OK;
    }
    return members[0].H.dtype == CG_F64 ? run_t<double>(ctx, nmembers, members, params, nsteps, t_host)
                                        : run_t<float>(ctx, nmembers, members, params, nsteps, t_host);
}

extern "C" int cg_sia_ensemble_tape_bytes(int nmembers, const cg_sia_member* members, int nsteps, size_t* bytes) {
    if (nmembers < 1 || !members || !bytes || nsteps < 0) return CG_ERR_ARG;
    const int dt = members[0].H.dtype;
    if (dt != CG_F32 && dt != CG_F64) return CG_ERR_ARG;
    const EnsTape et = ens_tape_layout(nmembers, members, dt == CG_F64 ? 8 : 4);
    *bytes = 256 + (size_t)nsteps * et.step_bytes;
    return CG_OK;
}

extern "C" int cg_sia_ensemble_run_taped(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                         const cg_sia_params* params, int nsteps, void* tape, size_t tape_bytes,
                                         double* t_host) {
    int rc = check_ensemble(ctx, nmembers, members, params, "sia_ensemble_run_taped");
    if (rc) return rc;
    if (nsteps < 1) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run_taped: nsteps < 1");
    size_t need = 0;
    cg_sia_ensemble_tape_bytes(nmembers, members, nsteps, &need);
    if (!tape || tape_bytes < need)
        return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run_taped: the tape holds %zu bytes, %d steps need %zu", tape_bytes,
                       nsteps, need);
    if (reinterpret_cast<uintptr_t>(tape) & 255)
        return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run_taped: the tape is not 256-byte aligned");
    cudaSetDevice(ctx->device);
    const int dt = members[0].H.dtype;
    EnsTapeHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    hd.magic = kEnsTapeMagic;
    hd.dtype = dt;
    hd.nm = nmembers;
    hd.nsteps = nsteps;
    hd.step_bytes = ens_tape_layout(nmembers, members, dt == CG_F64 ? 8 : 4).step_bytes;
    hd.hash = ens_tape_hash(nmembers, members, params);
    CG_CUDA(ctx, cudaMemcpyAsync(tape, &hd, sizeof(hd), cudaMemcpyHostToDevice, ctx->stream));
    char* tp = static_cast<char*>(tape);
    return dt == CG_F64 ? run_t<double>(ctx, nmembers, members, params, nsteps, t_host, tp)
                        : run_t<float>(ctx, nmembers, members, params, nsteps, t_host, tp);
}

extern "C" int cg_sia_ensemble_adjoint_run(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                           const cg_sia_params* params, const void* tape, size_t tape_bytes,
                                           const cg_field* lam, const cg_field* work, double* dJ) {
    int rc = check_ensemble(ctx, nmembers, members, params, "sia_ensemble_adjoint_run");
    if (rc) return rc;
    if (!tape || !lam || !work) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: NULL argument");
    const int dt = members[0].H.dtype;
    for (int m = 0; m < nmembers; ++m) {
        const cg_field& H = members[m].H;
        if ((rc = cg_check_field(ctx, &members[m].grid, lam[m], dt, 0, "lambda"))) return rc;
        if ((rc = cg_check_field(ctx, &members[m].grid, work[m], dt, 0, "work"))) return rc;
        if (lam[m].data == work[m].data) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: lambda and work alias (member %d)", m);
        for (const cg_field* f : {&lam[m], &work[m]})
            if (f->stride[1] != H.stride[1] || f->halo[0] != H.halo[0] || f->halo[1] != H.halo[1] || f->n[0] != H.n[0] ||
                f->n[1] != H.n[1])
                return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: lambda and work need H's layout (member %d)", m);
    }
    if (tape_bytes < sizeof(EnsTapeHeader)) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: the tape is too small");
    cudaSetDevice(ctx->device);
    EnsTapeHeader hd;
    CG_CUDA(ctx, cudaMemcpyAsync(&hd, tape, sizeof(hd), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hd.magic != kEnsTapeMagic)
        return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: no tape of cg_sia_ensemble_run_taped at this address");
    const EnsTape et = ens_tape_layout(nmembers, members, dt == CG_F64 ? 8 : 4);
    if (hd.dtype != dt || hd.nm != nmembers || hd.step_bytes != et.step_bytes ||
        hd.hash != ens_tape_hash(nmembers, members, params))
        return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: the tape was recorded for other members or parameters");
    if (hd.nsteps < 1 || tape_bytes < 256 + (size_t)hd.nsteps * et.step_bytes)
        return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_adjoint_run: the tape is shorter than its %d steps", hd.nsteps);
    return cg_sia_reverse_impl(ctx, nmembers, members, params, hd.nsteps, static_cast<const char*>(tape), lam, work, dJ);
}
