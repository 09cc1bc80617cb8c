// cg_sia.cu — shallow-ice flow (Chmy.jl examples/sia.jl:7-16,30-54,71-81).
#include "cg_common.cuh"
#include "cg_sia_kernels.cuh"

int cg_maxabs_collect(cg_ctx* ctx, int nfields, const cg_field* fields, double* out, int32_t* nonfinite);
void* cg_scratch(cg_ctx* ctx, int slot, size_t bytes, int* rc);

namespace {

template <class T>
struct SiaV {
    DF<T> H, B, qx, qy, D;
    T Gamma, As, beta, ela, m_max;
    T Gn2, Asn;  // Gamma (n+2) and As n, for the taped derivatives of D
    T idx, idy;
    int n;
};

template <class T>
__device__ __forceinline__ T S_at(const SiaV<T>& v, int i, int j) {
    return v.B(i, j, 0) + v.H(i, j, 0);
}

// ∇S at the cell's lower faces (a0, b0) and interpolated to the cell (ax, ay) (sia.jl:43-45)
template <class T>
__device__ __forceinline__ void grads_at(const SiaV<T>& v, int i, int j, T* a0, T* b0, T* ax, T* ay) {
    const T s = S_at(v, i, j);
    *a0 = (s - S_at(v, i - 1, j)) * v.idx;
    const T a1 = (S_at(v, i + 1, j) - s) * v.idx;
    *b0 = (s - S_at(v, i, j - 1)) * v.idy;
    const T b1 = (S_at(v, i, j + 1) - s) * v.idy;
    *ax = fma(T(0.5), a1 - *a0, *a0);
    *ay = fma(T(0.5), b1 - *b0, *b0);
}

// D = (Gamma H^(n+2) + As H^n) vmag(∇S)^(n-1) at cell (i, j) (sia.jl:43-49)
template <class T>
__device__ __forceinline__ T D_at(const SiaV<T>& v, int i, int j) {
    T a0, b0, ax, ay;
    grads_at(v, i, j, &a0, &b0, &ax, &ay);
    return cgsia::D_cell(v.H(i, j, 0), ax, ay, v.Gamma, v.As, v.n);
}

// The tape arrays of one step, in H's layout (cgsia::TapeArray; the masks one byte per cell),
// and its word block.
template <class T>
struct TapeV {
    DF<T> a[cgsia::kArrays];
    DF<unsigned char> fl;
    cgsia::TapeWords* w;
};

using cgsia::bits_of;

// update_q! over [1, n]^2 with D evaluated on the fly (the reference's FunctionField);
// optional max(interior D) into *dmax_bits (D >= 0, so the bit patterns order like values).
template <class T>
__global__ void sia_q_kernel(const SiaV<T> v, int nx, int ny, unsigned long long* dmax_bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const bool in = i <= nx && j <= ny;
    T dc = T(0);
    if (in) {
        dc = D_at(v, i, j);
        const T dl = D_at(v, i - 1, j), dd = D_at(v, i, j - 1);
        const T Dx = fma(T(0.5), dc - dl, dl);
        const T Dy = fma(T(0.5), dc - dd, dd);
        const T sc = S_at(v, i, j);
        v.qx(i, j, 0) = -Dx * ((sc - S_at(v, i - 1, j)) * v.idx);
        v.qy(i, j, 0) = -Dy * ((sc - S_at(v, i, j - 1)) * v.idy);
    }
    if (dmax_bits) cgsia::block_max_bits(in ? bits_of(dc) : 0ull, dmax_bits);
}

// D over cells [0, n]^2 into v.D and max over the interior [1, n]^2. TAPE: v.D is the tape's
// D, and the interior cells also record their lower faces' gradients and D's derivatives.
template <class T, bool TAPE = false>
__global__ void sia_D_kernel(const SiaV<T> v, int nx, int ny, unsigned long long* dmax_bits, const TapeV<T> tp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = i <= nx && j <= ny;
    T d = T(0);
    if (in) {
        T a0, b0, ax, ay;
        grads_at(v, i, j, &a0, &b0, &ax, &ay);
        const T h = v.H(i, j, 0);
        if (TAPE) {
            using namespace cgsia;
            T dh, ex, ey, gf;
            d = D_and_factors(h, ax, ay, v.Gamma, v.As, v.Gn2, v.Asn, v.n, &dh, &ex, &ey, &gf);
            if (i >= 1 && j >= 1) {
                tp.a[kGX](i, j, 0) = a0;
                tp.a[kGY](i, j, 0) = b0;
                tp.a[kDH](i, j, 0) = dh;
                tp.a[kEX](i, j, 0) = ex;
                tp.a[kEY](i, j, 0) = ey;
                tp.a[kGF](i, j, 0) = gf;
            }
        } else {
            d = cgsia::D_cell(h, ax, ay, v.Gamma, v.As, v.n);
        }
        v.D(i, j, 0) = d;
    }
    cgsia::block_max_bits(in && i >= 1 && j >= 1 ? bits_of(d) : 0ull, dmax_bits);
}

// update_q! from the precomputed D (same arithmetic as sia_q_kernel).
template <class T>
__global__ void sia_q_from_D_kernel(const SiaV<T> v, int nx, int ny) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx || j > ny) return;
    const T dc = v.D(i, j, 0), dl = v.D(i - 1, j, 0), dd = v.D(i, j - 1, 0);
    const T Dx = fma(T(0.5), dc - dl, dl);
    const T Dy = fma(T(0.5), dc - dd, dd);
    const T sc = S_at(v, i, j);
    v.qx(i, j, 0) = -Dx * ((sc - S_at(v, i - 1, j)) * v.idx);
    v.qy(i, j, 0) = -Dy * ((sc - S_at(v, i, j - 1)) * v.idy);
}

// update_H! over [1, n]^2; dt from a scalar or from device memory. TAPE: also W, the two
// masks, and the first interior cell where D attains the step's maximum.
template <class T, bool TAPE = false>
__global__ void sia_H_kernel(const SiaV<T> v, int nx, int ny, T dt_scalar, const double* dt_dev, const TapeV<T> tp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx || j > ny) return;
    const T dt = dt_dev ? (T)*dt_dev : dt_scalar;
    const T h = v.H(i, j, 0);
    const T x = v.beta * (S_at(v, i, j) - v.ela);
    const T m = fmin(x, v.m_max);
    T dv = (v.qx(i + 1, j, 0) - v.qx(i, j, 0)) * v.idx;
    dv = dv + (v.qy(i, j + 1, 0) - v.qy(i, j, 0)) * v.idy;
    const T W = -dv + m;
    const T u = h + dt * W;
    v.H(i, j, 0) = fmax(u, T(0.0));
    if (TAPE) {
        tp.a[cgsia::kW](i, j, 0) = W;
        tp.fl(i, j, 0) = (unsigned char)((u > T(0) ? 1 : 0) + (x < v.m_max ? 2 : 0));
        if (bits_of(v.D(i, j, 0)) == tp.w->dmax) atomicMin(&tp.w->arg, (unsigned long long)((long)j * (nx + 2) + i));
    }
}

// Δt = min(min(Δ)^2 / max(D) / cfl, dt_max); t += Δt; reset the max slot for the next step.
// `tw` (optional): the step's tape words.
template <class T>
__global__ void sia_dt_kernel(unsigned long long* dmax_bits, double* dt, double* t, double dx2, double cfl,
                              double dt_max, cgsia::TapeWords* tw) {
    const unsigned long long b = *dmax_bits;
    double dmax;
    if (sizeof(T) == 8) {
        dmax = __longlong_as_double((long long)b);
    } else {
        dmax = (double)__int_as_float((int)(unsigned)b);
    }
    // Julia: Δ^2 / maximum(D) / 4.1 in the grid type
    const T v = (T)dx2 / (T)dmax / (T)cfl;
    double d = fmin((double)v, dt_max);
    bool capped = !((double)v < dt_max);
    if (!(dmax > 0.0)) {
        d = dt_max;
        capped = true;
    }
    *dt = d;
    *t = *t + d;
    if (tw) {
        tw->dmax = b;
        tw->arg = ~0ull;
        tw->dt = d;
        tw->capped = capped ? 1.0 : 0.0;
    }
    *dmax_bits = 0ull;
}

template <class T>
SiaV<T> make_view(const cg_grid* g, const cg_field* H, const cg_field* B, const cg_field* q, const cg_sia_params* p,
                  void* D) {
    SiaV<T> v;
    std::memset(&v, 0, sizeof(v));
    v.H = cg_view<T>(*H);
    v.B = cg_view<T>(*B);
    if (q) {
        v.qx = cg_view<T>(q[0]);
        v.qy = cg_view<T>(q[1]);
    }
    if (D) {
        v.D = v.H;  // same layout as H
        v.D.p = static_cast<T*>(D) + cg_origin_offset(*H);
    }
    v.Gamma = (T)p->Gamma;
    v.As = (T)p->As;
    v.beta = (T)p->beta;
    v.ela = (T)p->ela;
    v.m_max = (T)p->m_max;
    v.Gn2 = v.Gamma * T(p->n + 2);
    v.Asn = v.As * T(p->n);
    v.idx = (T)g->inv_spacing[0];
    v.idy = (T)g->inv_spacing[1];
    v.n = p->n;
    return v;
}

int check_sia(cg_ctx* ctx, const cg_grid* g, const cg_field* H, const cg_field* B, const cg_field* q,
              const cg_sia_params* p) {
    int rc = cg_check_grid(ctx, g);
    if (rc) return rc;
    if (g->ndim != 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "sia: 2D grids only");
    if (!H || !B || !p) return cg_fail(ctx, CG_ERR_ARG, "sia: NULL argument");
    if ((rc = cg_check_field(ctx, g, *H, H->dtype, 0, "H"))) return rc;
    if ((rc = cg_check_field(ctx, g, *B, H->dtype, 0, "B"))) return rc;
    if (q) {
        if ((rc = cg_check_field(ctx, g, q[0], H->dtype, 1, "q.x"))) return rc;
        if ((rc = cg_check_field(ctx, g, q[1], H->dtype, 2, "q.y"))) return rc;
    }
    if (p->n < 1 || p->n > 16) return cg_fail(ctx, CG_ERR_ARG, "sia: Glen exponent %d not in 1..16", p->n);
    return CG_OK;
}

void sia_bcs(cg_bc* qb, cg_bc* hb) {
    std::memset(qb, 0, 2 * sizeof(cg_bc));
    qb[0].kind[0][0] = qb[0].kind[0][1] = CG_BC_DIRICHLET;
    qb[1].kind[1][0] = qb[1].kind[1][1] = CG_BC_DIRICHLET;
    std::memset(hb, 0, sizeof(cg_bc));
    hb->kind[0][0] = hb->kind[0][1] = hb->kind[1][0] = hb->kind[1][1] = CG_BC_NEUMANN;
}

template <class T>
int update_q_t(cg_ctx* ctx, const cg_grid* g, const cg_field* q, const cg_field* H, const cg_field* B,
               const cg_sia_params* p, double* dmax) {
    const SiaV<T> v = make_view<T>(g, H, B, q, p, nullptr);
    const dim3 block(32, 8), grid(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8));
    if (dmax) CG_CUDA(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    sia_q_kernel<T><<<grid, block, 0, ctx->stream>>>(v, g->n[0], g->n[1], dmax ? ctx->d_red : nullptr);
    CG_CHECK_LAUNCH(ctx);
    cg_bc qb[2], hb;
    sia_bcs(qb, &hb);
    int rc = cg_bc_apply_impl(ctx, g, 2, q, qb);
    if (rc) return rc;
    if (dmax) {
        cg_field probe = *H;  // dtype of the reduction slot
        double m;
        return cg_maxabs_collect(ctx, 1, &probe, &m, nullptr) ? CG_ERR_CUDA : ((*dmax = m), CG_OK);
    }
    return CG_OK;
}

template <class T>
int update_H_t(cg_ctx* ctx, const cg_grid* g, const cg_field* H, const cg_field* q, const cg_field* B, double dt,
               const cg_sia_params* p) {
    const SiaV<T> v = make_view<T>(g, H, B, q, p, nullptr);
    const dim3 block(32, 8), grid(cg_div_up(g->n[0], 32), cg_div_up(g->n[1], 8));
    sia_H_kernel<T><<<grid, block, 0, ctx->stream>>>(v, g->n[0], g->n[1], (T)dt, nullptr, TapeV<T>{});
    CG_CHECK_LAUNCH(ctx);
    cg_bc qb[2], hb;
    sia_bcs(qb, &hb);
    return cg_bc_apply_impl(ctx, g, 1, H, &hb);
}

template <class T>
int run_t(cg_ctx* ctx, const cg_grid* g, const cg_field* H, const cg_field* B, const cg_field* q,
          const cg_sia_params* p, int nsteps, double* t_host, char* tape = nullptr) {
    // scratch: D (same padded layout as H) + 3 words (max bits, dt, t)
    long cnt = 1;
    for (int d = 0; d < 2; ++d) cnt *= (H->n[d] + 4L * H->halo[d]);
    cnt = std::max<long>(cnt, (long)H->stride[1] * (H->n[1] + 4L * H->halo[1]));
    int rc = CG_OK;
    char* base = static_cast<char*>(cg_scratch(ctx, 1, cnt * sizeof(T) + 256 + 64, &rc));
    if (rc) return rc;
    unsigned long long* words = reinterpret_cast<unsigned long long*>(base + ((cnt * sizeof(T) + 255) & ~255L));
    double* dt = reinterpret_cast<double*>(words + 1);
    double* t = reinterpret_cast<double*>(words + 2);
    CG_CUDA(ctx, cudaMemsetAsync(words, 0, 3 * sizeof(unsigned long long), ctx->stream));
    const SiaV<T> v = make_view<T>(g, H, B, q, p, base);
    const int nx = g->n[0], ny = g->n[1];
    const dim3 block(32, 8);
    const dim3 gD(cg_div_up(nx + 1, 32), cg_div_up(ny + 1, 8)), gI(cg_div_up(nx, 32), cg_div_up(ny, 8));
    const double dx = std::min(g->spacing[0], g->spacing[1]);
    const double dx2 = (double)((T)dx * (T)dx);
    cg_bc qb[2], hb;
    sia_bcs(qb, &hb);
    std::string key = "sia_run";
    cg_key_add(key, *g);
    cg_key_add(key, *H);
    cg_key_add(key, *B);
    cg_key_add(key, q[0]);
    cg_key_add(key, q[1]);
    cg_key_add(key, *p);
    cg_key_add(key, nsteps);
    cg_key_add(key, base);
    cg_key_add(key, tape);
    const cgsia::TapeGeom tg = cgsia::tape_geom(*H, sizeof(T));
    rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int s = 0; s < nsteps; ++s) {
            SiaV<T> vs = v;
            TapeV<T> tp{};
            if (tape) {
                char* sb = tape + 256 + (size_t)s * tg.step_bytes;
                tp.w = reinterpret_cast<cgsia::TapeWords*>(sb);
                for (int k = 0; k < cgsia::kArrays; ++k) {
                    tp.a[k] = v.H;
                    tp.a[k].p = reinterpret_cast<T*>(sb + 256 + (size_t)k * tg.abytes) + cg_origin_offset(*H);
                }
                tp.fl.p = reinterpret_cast<unsigned char*>(sb + 256 + (size_t)cgsia::kFL * tg.abytes) + cg_origin_offset(*H);
                tp.fl.s1 = v.H.s1;
                tp.fl.s2 = v.H.s2;
                vs.D = tp.a[cgsia::kD];
                sia_D_kernel<T, true><<<gD, block, 0, st>>>(vs, nx, ny, words, tp);
            } else {
                sia_D_kernel<T><<<gD, block, 0, st>>>(vs, nx, ny, words, tp);
            }
            sia_q_from_D_kernel<T><<<gI, block, 0, st>>>(vs, nx, ny);
            CG_CHECK_LAUNCH(ctx);
            int r = cg_bc_apply_impl(ctx, g, 2, q, qb);
            if (r) return r;
            sia_dt_kernel<T><<<1, 1, 0, st>>>(words, dt, t, dx2, p->cfl, p->dt_max, tp.w);
            if (tape)
                sia_H_kernel<T, true><<<gI, block, 0, st>>>(vs, nx, ny, T(0), dt, tp);
            else
                sia_H_kernel<T><<<gI, block, 0, st>>>(vs, nx, ny, T(0), dt, tp);
            CG_CHECK_LAUNCH(ctx);
            r = cg_bc_apply_impl(ctx, g, 1, H, &hb);
            if (r) return r;
        }
        return (int)CG_OK;
    });
    if (rc) return rc;
    if (t_host) {
        CG_CUDA(ctx, cudaMemcpyAsync(t_host, t, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return CG_OK;
}

}  // namespace

extern "C" int cg_sia_update_q(cg_ctx* ctx, const cg_grid* grid, const cg_field* q, const cg_field* H,
                               const cg_field* B, const cg_sia_params* p, double* dmax_host) {
    int rc = check_sia(ctx, grid, H, B, q, p);
    if (rc) return rc;
    if (!q) return cg_fail(ctx, CG_ERR_ARG, "sia_update_q: q is NULL");
    cudaSetDevice(ctx->device);
    return H->dtype == CG_F64 ? update_q_t<double>(ctx, grid, q, H, B, p, dmax_host)
                              : update_q_t<float>(ctx, grid, q, H, B, p, dmax_host);
}

extern "C" int cg_sia_update_H(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* q,
                               const cg_field* B, double dt, const cg_sia_params* p) {
    int rc = check_sia(ctx, grid, H, B, q, p);
    if (rc) return rc;
    if (!q) return cg_fail(ctx, CG_ERR_ARG, "sia_update_H: q is NULL");
    cudaSetDevice(ctx->device);
    return H->dtype == CG_F64 ? update_H_t<double>(ctx, grid, H, q, B, dt, p)
                              : update_H_t<float>(ctx, grid, H, q, B, dt, p);
}

extern "C" int cg_sia_tape_bytes(const cg_grid* grid, const cg_field* H, int nsteps, size_t* bytes) {
    if (!grid || !H || !bytes || nsteps < 0) return CG_ERR_ARG;
    if (grid->ndim != 2 || (H->dtype != CG_F32 && H->dtype != CG_F64)) return CG_ERR_ARG;
    const cgsia::TapeGeom tg = cgsia::tape_geom(*H, H->dtype == CG_F64 ? 8 : 4);
    *bytes = 256 + (size_t)nsteps * tg.step_bytes;
    return CG_OK;
}

extern "C" int cg_sia_run_taped(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B,
                                const cg_field* q, const cg_sia_params* p, int nsteps, void* tape, size_t tape_bytes,
                                double* t_host) {
    int rc = check_sia(ctx, grid, H, B, q, p);
    if (rc) return rc;
    if (!q) return cg_fail(ctx, CG_ERR_ARG, "sia_run_taped: q is NULL");
    if (nsteps < 1) return cg_fail(ctx, CG_ERR_ARG, "sia_run_taped: nsteps < 1");
    if (p->cfl <= 0 || p->dt_max <= 0) return cg_fail(ctx, CG_ERR_ARG, "sia_run_taped: cfl and dt_max must be > 0");
    size_t need = 0;
    cg_sia_tape_bytes(grid, H, nsteps, &need);
    if (!tape || tape_bytes < need)
        return cg_fail(ctx, CG_ERR_ARG, "sia_run_taped: the tape holds %zu bytes, %d steps need %zu", tape_bytes, nsteps, need);
    if (reinterpret_cast<uintptr_t>(tape) & 255) return cg_fail(ctx, CG_ERR_ARG, "sia_run_taped: the tape is not 256-byte aligned");
    cudaSetDevice(ctx->device);
    const size_t elem = H->dtype == CG_F64 ? 8 : 4;
    const cgsia::TapeGeom tg = cgsia::tape_geom(*H, elem);
    cgsia::TapeHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    hd.magic = cgsia::kTapeMagic;
    hd.dtype = H->dtype;
    hd.nx = grid->n[0];
    hd.ny = grid->n[1];
    hd.nsteps = nsteps;
    hd.stride0 = H->stride[0];
    hd.stride1 = H->stride[1];
    hd.halo0 = H->halo[0];
    hd.halo1 = H->halo[1];
    hd.n0 = H->n[0];
    hd.n1 = H->n[1];
    hd.cnt = (long long)tg.cnt;
    hd.step_bytes = (long long)tg.step_bytes;
    hd.Gamma = p->Gamma;
    hd.As = p->As;
    hd.beta = p->beta;
    hd.ela = p->ela;
    hd.m_max = p->m_max;
    hd.cfl = p->cfl;
    hd.dt_max = p->dt_max;
    hd.n = p->n;
    CG_CUDA(ctx, cudaMemcpyAsync(tape, &hd, sizeof(hd), cudaMemcpyHostToDevice, ctx->stream));
    char* tp = static_cast<char*>(tape);
    return H->dtype == CG_F64 ? run_t<double>(ctx, grid, H, B, q, p, nsteps, t_host, tp)
                              : run_t<float>(ctx, grid, H, B, q, p, nsteps, t_host, tp);
}

extern "C" int cg_sia_run(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B, const cg_field* q,
                          const cg_sia_params* p, int nsteps, double* t_host) {
    int rc = check_sia(ctx, grid, H, B, q, p);
    if (rc) return rc;
    if (!q) return cg_fail(ctx, CG_ERR_ARG, "sia_run: q is NULL");
    if (nsteps < 0) return cg_fail(ctx, CG_ERR_ARG, "sia_run: nsteps < 0");
    if (p->cfl <= 0 || p->dt_max <= 0) return cg_fail(ctx, CG_ERR_ARG, "sia_run: cfl and dt_max must be > 0");
    cudaSetDevice(ctx->device);
    if (nsteps == 0) {
        if (t_host) *t_host = 0.0;
        return CG_OK;
    }
    return H->dtype == CG_F64 ? run_t<double>(ctx, grid, H, B, q, p, nsteps, t_host)
                              : run_t<float>(ctx, grid, H, B, q, p, nsteps, t_host);
}
