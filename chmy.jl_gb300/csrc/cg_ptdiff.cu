// cg_ptdiff.cu — pseudo-transient variable-coefficient diffusion (implicit step solved by
// damped PT iterations; flux in Chmy's ∂k∂ form, src/GridOperators/partial_derivatives.jl:14-21).
#include "cg_common.cuh"


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

template <class T, int ND>
int launch_q(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    const dim3 b = block_for<ND>();
    ptdiff_q_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(make_pv<T>(g, f, p), g->n[0] + 1,
                                                                         ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int launch_C(cg_ctx* ctx, const cg_grid* g, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    const dim3 b = block_for<ND>();
    ptdiff_C_kernel<T, ND><<<range_grid<ND>(g, b), b, 0, ctx->stream>>>(make_pv<T>(g, f, p), g->n[0] + 1,
                                                                         ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

#define PDISPATCH(fn, dtype, nd, ...)                                                                     \
    ((dtype) == CG_F64 ? ((nd) == 1 ? fn<double, 1>(__VA_ARGS__)                                         \
                                    : (nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__)) \
                       : ((nd) == 1 ? fn<float, 1>(__VA_ARGS__)                                          \
                                    : (nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

// Bytes from the first to the last element of the padded field (pitched rows included).
size_t padded_bytes(const cg_field& f) {
    size_t span = 1;
    for (int d = 0; d < f.ndim; ++d) span += (size_t)(f.n[d] + 4 * f.halo[d] - 1) * (size_t)f.stride[d];
    return span * (f.dtype == CG_F64 ? 8 : 4);
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
    const size_t cbytes = padded_bytes(f->C);
    const int dtype = f->C.dtype, nd = grid->ndim;
    return cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int s = 0; s < nsteps; ++s) {
            // update_old: C_old <- C (whole padded array)
            CG_CUDA(ctx, cudaMemcpyAsync(f->C_old.data, f->C.data, cbytes, cudaMemcpyDeviceToDevice, st));
            for (int it = 0; it < npt; ++it) {
                int r = PDISPATCH(launch_q, dtype, nd, ctx, grid, f, p);
                if (r) return r;
                r = PDISPATCH(launch_C, dtype, nd, ctx, grid, f, p);
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
