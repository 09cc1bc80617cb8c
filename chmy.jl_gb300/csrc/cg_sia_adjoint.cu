// cg_sia_adjoint.cu — reverse step of the shallow-ice time loop (examples/sia.jl:71-81, the
// flux of cg_sia_run): the adjoint state and the gradient of a misfit with respect to the
// flux factor Gamma and the equilibrium-line altitude ela.
//
// One forward step (interior cells c, faces f between cells f-1 and f):
//   S = B + H,  D_c = (Gamma h^(n+2) + As h^n) V_c^((n-1)/2),  V_c = ax_c^2 + ay_c^2,
//   ax_c = lerp(gx_c, gx_c+1), gx_f = (S_f - S_f-1)/dx,
//   qx_f = -lerp(D)_f gx_f on faces 2..n, 0 on faces 1 and n+1 (bc! Dirichlet); y likewise,
//   dt = min(dx^2 / max_c D_c / cfl, dt_max),
//   W_c = -divg(q)_c + M_c,  M_c = min(beta (S_c - ela), m_max),
//   H'_c = max(H_c + dt W_c, 0), then bc! copies the first interior cells into the ghost layer.
// For lambda = dJ/dH' at the interior cells, the reverse step gives dJ/dH at the interior
// cells, with the ghost cells' adjoints folded into the cells they copy, and adds this step's
// dJ/dGamma and dJ/dela. With mu_c = lambda_c [H_c + dt W_c > 0] and mM_c = [beta (S_c - ela)
// < m_max]:
// - direct: dJ/dH_c += mu_c (1 + dt beta mM_c); dJ/dela -= sum mu_c dt beta mM_c.
// - time step: dJ/ddt = sum mu_c W_c. When dt is not capped, dt = dx^2/(cfl Dmax), so
//   dJ/dD_c* gains -dJ/ddt dt / Dmax at the cell c* where D attains its maximum.
// - fluxes: dJ/dqx_f = dt/dx (mu_f - mu_f-1) on faces 2..n. Each such face adds -gx_f/2 of it
//   to dJ/dD of both its cells, and -lerp(D)_f/dx times it to dJ/dS of its upper cell, or
//   +lerp(D)_f/dx to its lower cell.
// - D: dJ/dH_c += dJ/dD_c dD/dh; dJ/dGamma += dJ/dD_c h^(n+2) V^((n-1)/2); with
//   dJ/dV_c = dJ/dD_c dD/dV, cell c's S neighbours gain -/+ dJ/dV_c ax_c/dx (x) and
//   ay_c/dy (y).
// - S = B + H: dJ/dH_c += dJ/dS_c at every cell; the ghost cells' terms go to the interior
//   cells they copy (corners are never read).
// The kernels gather instead of scatter: each cell sums the terms of its own faces and
// neighbours, so no two threads write one address. The forward quantities are recomputed
// from H with the arithmetic of cg_sia_run, so the masks and Dmax match the forward step.
#include <cmath>
#include <cstddef>

#include "cg_common.cuh"
#include "cg_sia_kernels.cuh"

void* cg_scratch(cg_ctx* ctx, int slot, size_t bytes, int* rc);
int cg_sia_reverse_impl(cg_ctx* ctx, int nm, const cg_sia_member* ms, const cg_sia_params* ps, int nsteps,
                        const char* tape, const cg_field* lam, const cg_field* work, double* dJ);

namespace {

template <class T>
struct SiaAdj {
    DF<T> H, B, D, lam, out, mu, lo, pax, pay;
    T Gamma, As, beta, ela, m_max, idx, idy;
    int n, nx, ny;
};

// device words: the step's Dmax bits, argmax index, dt, capped flag and dJ/ddt (reset every
// step), then dJ/dGamma and dJ/dela accumulated over the steps until a call reads them
struct SiaWords {
    unsigned long long dmax;
    unsigned long long arg;
    double dt;
    double capped;
    double dJdt;
    double gG;
    double gE;
};

template <class T>
__device__ __forceinline__ T S_of(const SiaAdj<T>& v, int i, int j) {
    return v.B(i, j, 0) + v.H(i, j, 0);
}

template <class T>
__device__ __forceinline__ void grads(const SiaAdj<T>& v, int i, int j, T* ax, T* ay) {
    const T s = S_of(v, i, j);
    const T a0 = (s - S_of(v, i - 1, j)) * v.idx;
    const T a1 = (S_of(v, i + 1, j) - s) * v.idx;
    const T b0 = (s - S_of(v, i, j - 1)) * v.idy;
    const T b1 = (S_of(v, i, j + 1) - s) * v.idy;
    *ax = fma(T(0.5), a1 - a0, a0);
    *ay = fma(T(0.5), b1 - b0, b0);
}

// x-face flux at face f of row j, as cg_sia_run leaves it after bc!(q). The product is rounded
// on its own (rmul), as the forward stores it: fused into the divergence's subtraction it would
// round differently, and H + dt W could then fall on the other side of the max(., 0) kink.
template <class T>
__device__ __forceinline__ T qx_at(const SiaAdj<T>& v, int f, int j) {
    if (f <= 1 || f >= v.nx + 1) return T(0);
    const T dc = v.D(f, j, 0), dl = v.D(f - 1, j, 0);
    return cgk::rmul(-fma(T(0.5), dc - dl, dl), (S_of(v, f, j) - S_of(v, f - 1, j)) * v.idx);
}
template <class T>
__device__ __forceinline__ T qy_at(const SiaAdj<T>& v, int i, int f) {
    if (f <= 1 || f >= v.ny + 1) return T(0);
    const T dc = v.D(i, f, 0), dl = v.D(i, f - 1, 0);
    return cgk::rmul(-fma(T(0.5), dc - dl, dl), (S_of(v, i, f) - S_of(v, i, f - 1)) * v.idy);
}

// D at the interior cells and its maximum (the forward's Dmax)
template <class T>
__global__ void adj_D_kernel(const SiaAdj<T> v, SiaWords* w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const bool in = i <= v.nx && j <= v.ny;
    T d = T(0);
    if (in) {
        T ax, ay;
        grads(v, i, j, &ax, &ay);
        d = cgsia::D_cell(v.H(i, j, 0), ax, ay, v.Gamma, v.As, v.n);
        v.D(i, j, 0) = d;
    }
    cgk::block_max_bits(in ? cgk::bits_of(d) : 0ull, &w->dmax);
}

// dt exactly as the forward computes it, whether it is capped, and the argmax slot's reset
template <class T>
__global__ void adj_dt_kernel(SiaWords* w, double dx2, double cfl, double dt_max) {
    const unsigned long long b = w->dmax;
    const double dmax = sizeof(T) == 8 ? __longlong_as_double((long long)b) : (double)__int_as_float((int)(unsigned)b);
    const T q = (T)dx2 / (T)dmax / (T)cfl;
    double d = fmin((double)q, dt_max);
    bool capped = !((double)q < dt_max);
    if (!(dmax > 0.0)) {
        d = dt_max;
        capped = true;
    }
    w->dt = d;
    w->capped = capped ? 1.0 : 0.0;
    w->arg = ~0ull;
    w->dJdt = 0.0;
}

// the first interior cell (lowest linear index) where D equals the maximum
template <class T>
__global__ void adj_arg_kernel(const SiaAdj<T> v, SiaWords* w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    if (cgk::bits_of(v.D(i, j, 0)) == w->dmax) atomicMin(&w->arg, (unsigned long long)((long)j * (v.nx + 2) + i));
}

using cgsia::block_sum;

// Sums over the blocks' partials in a fixed order (one block of 256 threads): for each of the
// `narr` arrays part[k][0..nblocks), dst_k = (acc_k ? dst_k : 0) + sum_b part[k][b].
// The per-block partials and this ordered sum keep the gradients reproducible bit for bit,
// where atomic adds would round in arrival order.
__global__ void adj_sum_kernel(const double* part, int nblocks, int narr, double* dst0, double* dst1, int acc0,
                               int acc1) {
    __shared__ double red[256];
    for (int k = 0; k < narr; ++k) {
        const double* a = part + (size_t)k * nblocks;
        double x = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x += a[b];
        red[threadIdx.x] = x;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            double* d = k == 0 ? dst0 : dst1;
            const int acc = k == 0 ? acc0 : acc1;
            if (d) *d = acc ? *d + red[0] : red[0];
        }
        __syncthreads();
    }
}

// mu, the direct term into lo, and the step's dJ/ddt and dJ/dela partial sums per block
template <class T>
__global__ void adj_mu_kernel(const SiaAdj<T> v, SiaWords* w, double* part, int nblocks) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const bool in = i <= v.nx && j <= v.ny;
    double sdt = 0.0, sela = 0.0;
    if (in) {
        const T dt = (T)w->dt;
        const T h = v.H(i, j, 0);
        const T x = v.beta * (S_of(v, i, j) - v.ela);
        const T m = fmin(x, v.m_max);
        T dv = (qx_at(v, i + 1, j) - qx_at(v, i, j)) * v.idx;
        dv = dv + (qy_at(v, i, j + 1) - qy_at(v, i, j)) * v.idy;
        const T W = -dv + m;
        const T u = h + dt * W;
        const T mu = u > T(0) ? v.lam(i, j, 0) : T(0);
        const T mM = x < v.m_max ? T(1) : T(0);
        v.mu(i, j, 0) = mu;
        v.lo(i, j, 0) = mu * (T(1) + dt * v.beta * mM);
        sdt = (double)(mu * W);
        sela = -(double)(mu * dt * v.beta * mM);
    }
    const double a = block_sum(sdt);
    const double b = block_sum(sela);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const int blk = blockIdx.x + gridDim.x * blockIdx.y;
        part[blk] = a;
        part[nblocks + blk] = b;
    }
}

// dJ/dD from the cell's faces (and the dt term at the argmax cell), then the D chain: lo +=
// dJ/dD dD/dh, the gradient parts dJ/dax, dJ/day, and the step's dJ/dGamma
template <class T>
__global__ void adj_D_back_kernel(const SiaAdj<T> v, SiaWords* w, double* part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const bool in = i <= v.nx && j <= v.ny;
    double sG = 0.0;
    if (in) {
        const T dt = (T)w->dt;
        const T dtx = dt * v.idx, dty = dt * v.idy;
        const T muc = v.mu(i, j, 0);
        T pD = T(0), pS = T(0);
        // x faces i (cell is upper) and i+1 (cell is lower); faces 1 and n+1 carry no flux
        if (i >= 2) {
            const T px = dtx * (muc - v.mu(i - 1, j, 0));
            const T dl = v.D(i - 1, j, 0), dc = v.D(i, j, 0);
            const T gx = (S_of(v, i, j) - S_of(v, i - 1, j)) * v.idx;
            pD += -T(0.5) * px * gx;
            pS += -fma(T(0.5), dc - dl, dl) * px * v.idx;
        }
        if (i + 1 <= v.nx) {
            const T px = dtx * (v.mu(i + 1, j, 0) - muc);
            const T dl = v.D(i, j, 0), dc = v.D(i + 1, j, 0);
            const T gx = (S_of(v, i + 1, j) - S_of(v, i, j)) * v.idx;
            pD += -T(0.5) * px * gx;
            pS += fma(T(0.5), dc - dl, dl) * px * v.idx;
        }
        if (j >= 2) {
            const T py = dty * (muc - v.mu(i, j - 1, 0));
            const T dl = v.D(i, j - 1, 0), dc = v.D(i, j, 0);
            const T gy = (S_of(v, i, j) - S_of(v, i, j - 1)) * v.idy;
            pD += -T(0.5) * py * gy;
            pS += -fma(T(0.5), dc - dl, dl) * py * v.idy;
        }
        if (j + 1 <= v.ny) {
            const T py = dty * (v.mu(i, j + 1, 0) - muc);
            const T dl = v.D(i, j, 0), dc = v.D(i, j + 1, 0);
            const T gy = (S_of(v, i, j + 1) - S_of(v, i, j)) * v.idy;
            pD += -T(0.5) * py * gy;
            pS += fma(T(0.5), dc - dl, dl) * py * v.idy;
        }
        // dt = dx^2 / (cfl Dmax) when not capped: the argmax cell carries dJ/dDmax
        if (w->capped == 0.0 && (unsigned long long)((long)j * (v.nx + 2) + i) == w->arg) {
            const unsigned long long b = w->dmax;
            const double dmax =
                sizeof(T) == 8 ? __longlong_as_double((long long)b) : (double)__int_as_float((int)(unsigned)b);
            pD += (T)(-w->dJdt * w->dt / dmax);
        }
        // D = (Gamma h^(n+2) + As h^n) V^((n-1)/2)
        T ax, ay;
        grads(v, i, j, &ax, &ay);
        const T h = v.H(i, j, 0);
        const T V = ax * ax + ay * ay;
        const int n = v.n;
        T vp = cgsia::pow_int(V, (n - 1) >> 1);
        if ((n - 1) & 1) vp = vp * sqrt(V);
        const T hn = cgsia::pow_int(h, n);
        const T A = hn * fma(v.Gamma, h * h, v.As);
        const T dDdh = (v.Gamma * T(n + 2) * h * h + v.As * T(n)) * (n >= 1 ? cgsia::pow_int(h, n - 1) : T(0)) * vp;
        T dDdV = T(0);
        if (n >= 3) {
            T vq = cgsia::pow_int(V, (n - 3) >> 1);
            if ((n - 3) & 1) vq = vq * sqrt(V);
            dDdV = A * T(0.5) * T(n - 1) * vq;
        } else if (n == 2 && V > T(0)) {
            dDdV = A * T(0.5) / sqrt(V);
        }
        v.lo(i, j, 0) = v.lo(i, j, 0) + pD * dDdh + pS;
        const T pV = pD * dDdV;
        v.pax(i, j, 0) = pV * T(2) * ax;
        v.pay(i, j, 0) = pV * T(2) * ay;
        sG = (double)(pD * hn * h * h * vp);
    }
    const double a = block_sum(sG);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[blockIdx.x + gridDim.x * blockIdx.y] = a;
}

// lambda_n: lo plus the S terms of the neighbours' D (ax_c = (S_c+1 - S_c-1)/(2 dx) up to
// rounding), with the ghost cells' terms folded into the interior cells they copy
template <class T>
__global__ void adj_out_kernel(const SiaAdj<T> v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > v.nx || j > v.ny) return;
    const T hx = T(0.5) * v.idx, hy = T(0.5) * v.idy;
    auto PX = [&](int a, int b) { return (a >= 1 && a <= v.nx) ? v.pax(a, b, 0) : T(0); };
    auto PY = [&](int a, int b) { return (b >= 1 && b <= v.ny) ? v.pay(a, b, 0) : T(0); };
    T r = v.lo(i, j, 0) + hx * (PX(i - 1, j) - PX(i + 1, j)) + hy * (PY(i, j - 1) - PY(i, j + 1));
    // ghost (0, j) copies (1, j): its S term is -hx pax(1, j); (n+1, j) copies (n, j): +hx pax(n, j)
    if (i == 1) r += -hx * v.pax(1, j, 0);
    if (i == v.nx) r += hx * v.pax(v.nx, j, 0);
    if (j == 1) r += -hy * v.pay(i, 1, 0);
    if (j == v.ny) r += hy * v.pay(i, v.ny, 0);
    v.out(i, j, 0) = r;
}

template <class T>
int adjoint_step_t(cg_ctx* ctx, const cg_grid* g, const cg_field* H, const cg_field* B, const cg_sia_params* p,
                   const cg_field* lam, const cg_field* lam_out, double* dJ) {
    // scratch slot 5: D, mu, lo, pax, pay (H's layout) and the words
    const size_t cnt = (size_t)H->stride[1] * (H->n[1] + 4 * H->halo[1]);
    const size_t abytes = (cnt * sizeof(T) + 255) & ~(size_t)255;
    int rc = CG_OK;
    const dim3 block(32, 8), grid(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8));
    const int nblocks = (int)(grid.x * grid.y);
    const size_t pbytes = ((size_t)nblocks * 3 * sizeof(double) + 255) & ~(size_t)255;
    char* base = static_cast<char*>(cg_scratch(ctx, 5, abytes * 5 + 256 + pbytes, &rc));
    if (rc) return rc;
    SiaAdj<T> v;
    std::memset(&v, 0, sizeof(v));
    v.H = cg_view<T>(*H);
    v.B = cg_view<T>(*B);
    v.lam = cg_view<T>(*lam);
    v.out = cg_view<T>(*lam_out);
    DF<T>* arr[5] = {&v.D, &v.mu, &v.lo, &v.pax, &v.pay};
    for (int a = 0; a < 5; ++a) {
        *arr[a] = v.H;
        arr[a]->p = reinterpret_cast<T*>(base + a * abytes) + cg_origin_offset(*H);
    }
    SiaWords* w = reinterpret_cast<SiaWords*>(base + 5 * abytes);
    double* part = reinterpret_cast<double*>(base + 5 * abytes + 256);  // [dJ/ddt | dJ/dela | dJ/dGamma] per block
    v.Gamma = (T)p->Gamma;
    v.As = (T)p->As;
    v.beta = (T)p->beta;
    v.ela = (T)p->ela;
    v.m_max = (T)p->m_max;
    v.idx = (T)g->inv_spacing[0];
    v.idy = (T)g->inv_spacing[1];
    v.n = p->n;
    v.nx = g->n[0];
    v.ny = g->n[1];
    const double dx = std::min(g->spacing[0], g->spacing[1]);
    const double dx2 = (double)((T)dx * (T)dx);
    // one graph per argument set: reset the step's words, then the reverse step's kernels
    std::string key = "sia_adjoint_step";
    cg_key_add(key, *g);
    cg_key_add(key, *H);
    cg_key_add(key, *B);
    cg_key_add(key, *lam);
    cg_key_add(key, *lam_out);
    cg_key_add(key, *p);
    cg_key_add(key, base);
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        CG_CUDA(ctx, cudaMemsetAsync(w, 0, offsetof(SiaWords, gG), st));
        adj_D_kernel<T><<<grid, block, 0, st>>>(v, w);
        adj_dt_kernel<T><<<1, 1, 0, st>>>(w, dx2, p->cfl, p->dt_max);
        adj_arg_kernel<T><<<grid, block, 0, st>>>(v, w);
        adj_mu_kernel<T><<<grid, block, 0, st>>>(v, w, part, nblocks);
        adj_sum_kernel<<<1, 256, 0, st>>>(part, nblocks, 2, &w->dJdt, &w->gE, 0, 1);
        adj_D_back_kernel<T><<<grid, block, 0, st>>>(v, w, part + 2 * (size_t)nblocks);
        adj_sum_kernel<<<1, 256, 0, st>>>(part + 2 * (size_t)nblocks, nblocks, 1, &w->gG, nullptr, 1, 0);
        adj_out_kernel<T><<<grid, block, 0, st>>>(v);
        CG_CHECK_LAUNCH(ctx);
        return (int)CG_OK;
    });
    if (rc) return rc;
    if (dJ) {  // hand the accumulated sums over and start again from zero
        double acc[2];
        CG_CUDA(ctx, cudaMemcpyAsync(acc, &w->gG, sizeof(acc), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        CG_CUDA(ctx, cudaMemsetAsync(&w->gG, 0, sizeof(acc), ctx->stream));
        dJ[0] += acc[0];
        dJ[1] += acc[1];
    }
    return CG_OK;
}

// ---- reverse sweep over a tape -----------------------------------------------------------
//
// The forward quantities come from the tape that cg_sia_run_taped wrote, so a reverse step
// recomputes nothing. The sweep is the ensemble's (cg_sia_reverse_impl) with one member: a
// single-member tape has the same step blocks.
bool same_layout(const cg_field& a, const cgsia::TapeHeader& h) {
    return a.stride[0] == h.stride0 && a.stride[1] == h.stride1 && a.halo[0] == h.halo0 && a.halo[1] == h.halo1 &&
           a.n[0] == h.n0 && a.n[1] == h.n1;
}

}  // namespace

extern "C" int cg_sia_adjoint_run(cg_ctx* ctx, const cg_grid* grid, const cg_sia_params* p, const void* tape,
                                  size_t tape_bytes, const cg_field* lam, const cg_field* work, double* dJ) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "sia_adjoint_run: ctx is NULL");
    if (!grid || !p || !tape || !lam || !work) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: NULL argument");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (grid->ndim != 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "sia_adjoint_run: 2D grids only");
    const int dt = lam->dtype;
    if ((rc = cg_check_field(ctx, grid, *lam, dt, 0, "lambda"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *work, dt, 0, "work"))) return rc;
    if (lam->data == work->data) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: lambda and work alias");
    if (tape_bytes < sizeof(cgsia::TapeHeader)) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: the tape is too small");
    cudaSetDevice(ctx->device);
    cgsia::TapeHeader hd;
    CG_CUDA(ctx, cudaMemcpyAsync(&hd, tape, sizeof(hd), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hd.magic != cgsia::kTapeMagic) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: no tape of cg_sia_run_taped at this address");
    if (hd.dtype != dt || hd.nx != grid->n[0] || hd.ny != grid->n[1])
        return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: the tape was recorded for another grid or type");
    if (!same_layout(*lam, hd) || !same_layout(*work, hd))
        return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: lambda and work need the layout of the taped H");
    if (hd.Gamma != p->Gamma || hd.As != p->As || hd.beta != p->beta || hd.ela != p->ela || hd.m_max != p->m_max ||
        hd.cfl != p->cfl || hd.dt_max != p->dt_max || hd.n != p->n)
        return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: the parameters differ from the taped run's");
    if (hd.nsteps < 1 || tape_bytes < 256 + (size_t)hd.nsteps * (size_t)hd.step_bytes)
        return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_run: the tape is shorter than its %d steps", hd.nsteps);
    cg_sia_member mem;
    std::memset(&mem, 0, sizeof(mem));
    mem.grid = *grid;
    mem.H = *lam;  // the taped H's layout
    return cg_sia_reverse_impl(ctx, 1, &mem, p, hd.nsteps, static_cast<const char*>(tape), lam, work, dJ);
}

extern "C" int cg_sia_adjoint_step(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B,
                                   const cg_sia_params* p, const cg_field* lam, const cg_field* lam_out, double* dJ) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "sia_adjoint_step: ctx is NULL");
    if (!grid || !H || !B || !p || !lam || !lam_out) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_step: NULL argument");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (grid->ndim != 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "sia_adjoint_step: 2D grids only");
    const int dt = H->dtype;
    if ((rc = cg_check_field(ctx, grid, *H, dt, 0, "H"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *B, dt, 0, "B"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *lam, dt, 0, "lambda"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *lam_out, dt, 0, "lambda_out"))) return rc;
    if (lam->data == lam_out->data) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_step: lambda and lambda_out alias");
    if (p->n < 1 || p->n > 16 || p->cfl <= 0 || p->dt_max <= 0) return cg_fail(ctx, CG_ERR_ARG, "sia_adjoint_step: bad parameters");
    cudaSetDevice(ctx->device);
    return dt == CG_F64 ? adjoint_step_t<double>(ctx, grid, H, B, p, lam, lam_out, dJ)
                        : adjoint_step_t<float>(ctx, grid, H, B, p, lam, lam_out, dJ);
}
