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
    double dx2, cfl, dt_max;
    int n, nx, ny;
    int tiles_D, tiles_I;  // tiles of the [0, n] and [1, n] ranges (32 x 8 each)
};

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

template <class T>
__device__ __forceinline__ void ens_D_tile(const Member<T>* mem, const int* prefix, int nm, Words* w, int blk) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 1 + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x;
    const int j = (t / tx) * 8 + threadIdx.y;
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
        d = cgsia::D_cell(v.H(i, j, 0), ax, ay, v.Gamma, v.As, v.n);
        v.D(i, j, 0) = d;
        if (i >= 1 && j >= 1) {  // the lower faces' gradients, for the q kernel
            v.qx(i, j, 0) = a0;
            v.qy(i, j, 0) = b0;
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
    const int j = (t / tx) * 8 + threadIdx.y - 1;
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
    const int j = (t / tx) * 8 + threadIdx.y + 1;
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

template <class T>
__device__ __forceinline__ void ens_dt_member(const Member<T>* mem, Words* w, int m) {
    const Member<T>& v = mem[m];
    const unsigned long long b = w[m].dmax;
    const double dmax = sizeof(T) == 8 ? __longlong_as_double((long long)b) : (double)__int_as_float((int)(unsigned)b);
    const T q = (T)v.dx2 / (T)dmax / (T)v.cfl;
    double d = fmin((double)q, v.dt_max);
    if (!(dmax > 0.0)) d = v.dt_max;
    w[m].dt = d;
    w[m].t = w[m].t + d;
    w[m].dmax = 0ull;
}

template <class T>
__device__ __forceinline__ void ens_H_tile(const Member<T>* mem, const int* prefix, int nm, const Words* w, int blk) {
    const int m = find_member(prefix, nm, blk);
    const Member<T>& v = member_of(mem, m);
    const int t = blk - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x + 1;
    const int j = (t / tx) * 8 + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    const T dt = (T)w[m].dt;
    const T h = v.H(i, j, 0);
    // M = min(beta (S - ela), m_max) and H = max(H + dt (-divg q + M), 0), as std::min/max
    // (a NaN propagates as in the reference)
    T mb = v.beta * (v.S(i, j, 0) - v.ela);
    mb = v.m_max < mb ? v.m_max : mb;
    T dv = (v.qx(i + 1, j, 0) - v.qx(i, j, 0)) * v.idx;
    dv = dv + (v.qy(i, j + 1, 0) - v.qy(i, j, 0)) * v.idy;
    T hn = h + dt * (-dv + mb);
    hn = hn < T(0.0) ? T(0.0) : hn;
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

template <class T>
__global__ void ens_D_kernel(const Member<T>* mem, const int* prefix, int nm, Words* w) {
    ens_D_tile(mem, prefix, nm, w, blockIdx.x);
}
template <class T>
__global__ void ens_S_kernel(const Member<T>* mem, const int* prefix, int nm) {
    ens_S_tile(mem, prefix, nm, blockIdx.x);
}
template <class T>
__global__ void ens_q_kernel(const Member<T>* mem, const int* prefix, int nm) {
    ens_q_tile(mem, prefix, nm, blockIdx.x);
}
template <class T>
__global__ void ens_dt_kernel(const Member<T>* mem, int nm, Words* w) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nm) ens_dt_member(mem, w, m);
}
template <class T>
__global__ void ens_H_kernel(const Member<T>* mem, const int* prefix, int nm, const Words* w) {
    ens_H_tile(mem, prefix, nm, w, blockIdx.x);
}

// ---- one persistent launch for the whole run ------------------------------------------------
//
// The same tiles and arithmetic as the per-phase kernels: the resident blocks of a cooperative
// launch loop over each phase's tiles, with a grid barrier between the phases. Per step:
// D and the block maxima; barrier; Δt of every member (block 0) and the fluxes; barrier; the
// thickness; barrier. The barrier counts arrivals on one monotonic word. Its waits give up
// after two seconds (of the GPU's global timer) and set a timeout flag: the kernel then returns, and the
// host reports the error. A cooperative launch keeps every block resident, so the waits end.
struct GridBar {
    unsigned long long arrived;  // arrivals since the launch: barrier k completes at (k + 1) x blocks
    int timeout;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier `k` (0, 1, ...) of the launch: one relaxed add per block, then a bounded wait until
// all blocks have added. Nothing is reset, so the last block to arrive has no extra work.
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned nblocks, unsigned long long& k) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const unsigned long long target = (++k) * nblocks;
        __threadfence();
        atomicAdd(&b->arrived, 1ull);
        volatile unsigned long long* va = &b->arrived;
        const unsigned long long t0 = globaltimer_ns();
        while (*va < target) {
            if (globaltimer_ns() - t0 > 2000000000ull) {  // 2 s
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
                                                             Words* w, int nsteps, GridBar* bar) {
    const unsigned nb = gridDim.x;
    unsigned long long k = 0;
    for (int b = blockIdx.x; b < totS; b += nb) ens_S_tile(mem, pS, nm, b);
    if (!grid_barrier(bar, nb, k)) return;
    for (int s = 0; s < nsteps; ++s) {
        for (int b = blockIdx.x; b < totD; b += nb) ens_D_tile(mem, pD, nm, w, b);
        if (!grid_barrier(bar, nb, k)) return;
        if (blockIdx.x == 0)
            for (int m = threadIdx.x + blockDim.x * threadIdx.y; m < nm; m += blockDim.x * blockDim.y)
                ens_dt_member(mem, w, m);
        for (int b = blockIdx.x; b < totI; b += nb) ens_q_tile(mem, pI, nm, b);
        if (!grid_barrier(bar, nb, k)) return;
        for (int b = blockIdx.x; b < totI; b += nb) ens_H_tile(mem, pI, nm, w, b);
        if (!grid_barrier(bar, nb, k)) return;
    }
}

template <class T>
int run_t(cg_ctx* ctx, int nm, const cg_sia_member* ms, const cg_sia_params* ps, int nsteps, double* t_host) {
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
    int totD = 0, totI = 0, totS = 0;
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
        v.idx = (T)s.grid.inv_spacing[0];
        v.idy = (T)s.grid.inv_spacing[1];
        const double dx = std::min(s.grid.spacing[0], s.grid.spacing[1]);
        v.dx2 = (double)((T)dx * (T)dx);
        v.cfl = p.cfl;
        v.dt_max = p.dt_max;
        v.n = p.n;
        v.nx = s.grid.n[0];
        v.ny = s.grid.n[1];
        v.tiles_D = cg_div_up(v.nx + 1, 32) * cg_div_up(v.ny + 1, 8);
        v.tiles_I = cg_div_up(v.nx, 32) * cg_div_up(v.ny, 8);
        totD += v.tiles_D;
        totI += v.tiles_I;
        totS += cg_div_up(v.nx + 3, 32) * cg_div_up(v.ny + 3, 8);
        pD[m] = totD;
        pI[m] = totI;
        pS[m] = totS;
    }
    Member<T>* dmem = reinterpret_cast<Member<T>*>(base + mem_off);
    int* dpD = reinterpret_cast<int*>(base + pD_off);
    int* dpI = reinterpret_cast<int*>(base + pI_off);
    int* dpS = reinterpret_cast<int*>(base + pS_off);
    Words* dw = reinterpret_cast<Words*>(base + w_off);
    CG_CUDA(ctx, cudaMemcpyAsync(dmem, hm.data(), nm * sizeof(Member<T>), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dpD, pD.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dpI, pI.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dpS, pS.data(), nm * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemsetAsync(dw, 0, nm * sizeof(Words), ctx->stream));
    const dim3 block(32, 8);
    static const int coop = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        return cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess ? v : 0;
    }();
    if (coop && cg_sia_persistent_enabled()) {
        // the whole run in one cooperative launch of the resident blocks
        static const int bps = [] {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ens_persistent_kernel<T>, 256, 0) != cudaSuccess) nb = 0;
            return nb;
        }();
        if (bps < 1) return cg_fail(ctx, CG_ERR_CUDA, "sia_ensemble_run: the persistent kernel does not fit on an SM");
        GridBar* bar = reinterpret_cast<GridBar*>(base + bar_off);
        CG_CUDA(ctx, cudaMemsetAsync(bar, 0, sizeof(GridBar), ctx->stream));
        const Member<T>* cmem = dmem;
        const int *cpD = dpD, *cpI = dpI, *cpS = dpS;
        int anm = nm, atD = totD, atI = totI, atS = totS, ans = nsteps;
        void* args[] = {&cmem, &cpD, &cpI, &cpS, &anm, &atD, &atI, &atS, &dw, &ans, &bar};
        CG_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)ens_persistent_kernel<T>, dim3(bps * ctx->num_sms), block,
                                                 args, 0, ctx->stream));
        int timed_out = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&timed_out, &bar->timeout, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (timed_out) return cg_fail(ctx, CG_ERR_TIMEOUT, "sia_ensemble_run: a grid barrier of the persistent kernel timed out");
    } else {
    std::string key = "sia_ensemble";
    cg_key_add(key, nm);
    cg_key_add(key, nsteps);
    cg_key_add(key, base);
    key.append(reinterpret_cast<const char*>(hm.data()), nm * sizeof(Member<T>));
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        ens_S_kernel<T><<<totS, block, 0, st>>>(dmem, dpS, nm);
        for (int s = 0; s < nsteps; ++s) {
            ens_D_kernel<T><<<totD, block, 0, st>>>(dmem, dpD, nm, dw);
            ens_q_kernel<T><<<totI, block, 0, st>>>(dmem, dpI, nm);
            ens_dt_kernel<T><<<cg_div_up(nm, 64), 64, 0, st>>>(dmem, nm, dw);
            ens_H_kernel<T><<<totI, block, 0, st>>>(dmem, dpI, nm, dw);
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

}  // namespace

extern "C" int cg_sia_ensemble_run(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                   const cg_sia_params* params, int nsteps, double* t_host) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "sia_ensemble_run: ctx is NULL");
    if (nmembers < 1 || !members || !params) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run: no members");
    if (nsteps < 0) return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run: nsteps < 0");
    const int dtype = members[0].H.dtype;
    for (int m = 0; m < nmembers; ++m) {
        const cg_sia_member& s = members[m];
        int rc = cg_check_grid(ctx, &s.grid);
        if (rc) return rc;
        if (s.grid.ndim != 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "sia_ensemble_run: member %d is not 2D", m);
        if ((rc = cg_check_field(ctx, &s.grid, s.H, dtype, 0, "H"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.B, dtype, 0, "B"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.q[0], dtype, 1, "q.x"))) return rc;
        if ((rc = cg_check_field(ctx, &s.grid, s.q[1], dtype, 2, "q.y"))) return rc;
        if (params[m].n < 1 || params[m].n > 16 || params[m].cfl <= 0 || params[m].dt_max <= 0)
            return cg_fail(ctx, CG_ERR_ARG, "sia_ensemble_run: bad parameters for member %d", m);
    }
    cudaSetDevice(ctx->device);
    if (nsteps == 0) {
        if (t_host)
            for (int m = 0; m < nmembers; ++m) t_host[m] = 0.0;
        return CG_OK;
    }
    return dtype == CG_F64 ? run_t<double>(ctx, nmembers, members, params, nsteps, t_host)
                           : run_t<float>(ctx, nmembers, members, params, nsteps, t_host);
}
