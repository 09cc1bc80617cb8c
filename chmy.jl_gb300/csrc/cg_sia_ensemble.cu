// cg_sia_ensemble.cu — an ensemble of independent shallow-ice solves of uneven grid sizes
// (examples/sia.jl:7-16,71-81 per member) advanced together: every phase of a time step is ONE
// launch over the tiles of all members (a per-member tile prefix table maps blocks to
// members), the adaptive Δt of every member is computed on the device, and the whole
// `nsteps` loop is replayed from one CUDA graph.
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
template <class T>
__device__ __forceinline__ const Member<T>& member_of(const Member<T>* mem, int m) {
    __shared__ __align__(16) unsigned long long words[(sizeof(Member<T>) + 7) / 8];
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
__global__ void ens_D_kernel(const Member<T>* mem, const int* prefix, int nm, Words* w) {
    const int m = find_member(prefix, nm, blockIdx.x);
    const Member<T>& v = member_of(mem, m);
    const int t = blockIdx.x - (m ? prefix[m - 1] : 0);
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
__global__ void ens_S_kernel(const Member<T>* mem, const int* prefix, int nm) {
    const int m = find_member(prefix, nm, blockIdx.x);
    const Member<T>& v = member_of(mem, m);
    const int t = blockIdx.x - (m ? prefix[m - 1] : 0);
    const int tx = (v.nx + 3 + 31) / 32;
    const int i = (t % tx) * 32 + threadIdx.x - 1;
    const int j = (t / tx) * 8 + threadIdx.y - 1;
    if (i > v.nx + 1 || j > v.ny + 1) return;
    v.S(i, j, 0) = v.B(i, j, 0) + v.H(i, j, 0);
}

template <class T>
__global__ void ens_q_kernel(const Member<T>* mem, const int* prefix, int nm) {
    const int m = find_member(prefix, nm, blockIdx.x);
    const Member<T>& v = member_of(mem, m);
    const int t = blockIdx.x - (m ? prefix[m - 1] : 0);
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
__global__ void ens_dt_kernel(const Member<T>* mem, int nm, Words* w) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nm) return;
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
__global__ void ens_H_kernel(const Member<T>* mem, const int* prefix, int nm, const Words* w) {
    const int m = find_member(prefix, nm, blockIdx.x);
    const Member<T>& v = member_of(mem, m);
    const int t = blockIdx.x - (m ? prefix[m - 1] : 0);
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
    std::string key = "sia_ensemble";
    cg_key_add(key, nm);
    cg_key_add(key, nsteps);
    cg_key_add(key, base);
    key.append(reinterpret_cast<const char*>(hm.data()), nm * sizeof(Member<T>));
    const dim3 block(32, 8);
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
