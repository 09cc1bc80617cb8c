// cg_stokes.cu — pseudo-transient viscoelastic Stokes kernels
// (Chmy.jl examples/stokes_2d_inc_ve_T.jl:11-60, examples/stokes_3d_inc_ve_T.jl:11-77).
#include "cg_common.cuh"

int cg_maxabs_enqueue(cg_ctx* ctx, int nfields, const cg_field* fields);
int cg_maxabs_collect(cg_ctx* ctx, int nfields, const cg_field* fields, double* out, int32_t* nonfinite);
int cg_stokes_solve_dc(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                       const cg_bc* bc_V, const cg_solve_opts* o, cg_solve_result* res);

#include "cg_march3d_tma.cuh"
#include "cg_stokes_kernels.cuh"

namespace {
using namespace cgk;

// ---- argument checks ---------------------------------------------------------------------------

inline int shear_mask(int nd, int c) {
    if (nd == 2) return c == 2 ? 0b11 : 0;
    switch (c) {
        case 3: return 0b011;
        case 4: return 0b101;
        case 5: return 0b110;
        default: return 0;
    }
}

enum { NEED_V = 1, NEED_TAU = 2, NEED_TAU_OLD = 4, NEED_P = 8, NEED_T = 16, NEED_TOLD = 32, NEED_QT = 64 };

int check_stokes(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, int need, int* dtype_out) {
    int rc = cg_check_grid(ctx, g);
    if (rc) return rc;
    if (!f) return cg_fail(ctx, CG_ERR_ARG, "stokes: fields is NULL");
    const int nd = g->ndim;
    if (nd < 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes: 2D and 3D grids only");
    const int nt = nd == 2 ? 3 : 6;
    const int dtype = (need & NEED_TAU) ? f->tau[0].dtype : f->T.dtype;
    *dtype_out = dtype;
    if (need & NEED_V)
        for (int d = 0; d < nd; ++d)
            if ((rc = cg_check_field(ctx, g, f->V[d], dtype, 1 << d, "V"))) return rc;
    if (need & NEED_TAU)
        for (int c = 0; c < nt; ++c)
            if ((rc = cg_check_field(ctx, g, f->tau[c], dtype, shear_mask(nd, c), "tau"))) return rc;
    if (need & NEED_TAU_OLD)
        for (int c = 0; c < nt; ++c)
            if ((rc = cg_check_field(ctx, g, f->tau_old[c], dtype, shear_mask(nd, c), "tau_old"))) return rc;
    if ((need & NEED_P) && (rc = cg_check_field(ctx, g, f->P, dtype, 0, "P"))) return rc;
    if ((need & NEED_T) && (rc = cg_check_field(ctx, g, f->T, dtype, 0, "T"))) return rc;
    if ((need & NEED_TOLD) && (rc = cg_check_field(ctx, g, f->T_old, dtype, 0, "T_old"))) return rc;
    if (need & NEED_QT)
        for (int d = 0; d < nd; ++d)
            if ((rc = cg_check_field(ctx, g, f->qT[d], dtype, 1 << d, "qT"))) return rc;
    // optional fields
    if (cg_present(f->divV) && (rc = cg_check_field(ctx, g, f->divV, dtype, 0, "divV"))) return rc;
    if (cg_present(f->eta) && (rc = cg_check_field(ctx, g, f->eta, dtype, 0, "eta"))) return rc;
    if (cg_present(f->inv_eta) && (rc = cg_check_field(ctx, g, f->inv_eta, dtype, 0, "inv_eta"))) return rc;
    for (int d = 0; d < nd; ++d) {
        if (cg_present(f->r_V[d]) && (rc = cg_check_field(ctx, g, f->r_V[d], dtype, 1 << d, "r_V"))) return rc;
        if (cg_present(f->rho_g[d]) && (rc = cg_check_field(ctx, g, f->rho_g[d], dtype, 1 << d, "rho_g")))
            return rc;
    }
    if (cg_present(f->r_V[0]))
        for (int d = 1; d < nd; ++d)
            if (!cg_present(f->r_V[d])) return cg_fail(ctx, CG_ERR_ARG, "r_V: all components or none");
    return CG_OK;
}

// The body force of every velocity component: an array rho_g[d], a device FunctionField
// p->rho_g_fn[d] of a known kind, or neither.
int check_body(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p) {
    for (int d = 0; d < 3; ++d) {
        const int k = p->rho_g_fn[d].kind;
        if (k < CG_FN_NONE || k > CG_FN_AFFINE) return cg_fail(ctx, CG_ERR_ARG, "rho_g_fn[%d]: unknown kind %d", d, k);
        if (k != CG_FN_NONE && d >= g->ndim) return cg_fail(ctx, CG_ERR_ARG, "rho_g_fn[%d]: the grid has %d dims", d, g->ndim);
        if (k != CG_FN_NONE && cg_present(f->rho_g[d]))
            return cg_fail(ctx, CG_ERR_ARG, "rho_g[%d]: an array and a function were both given", d);
    }
    return CG_OK;
}

// Precomputed viscosity arrays of a solve (dense Center layout, halo 1, in the field type):
// [inv_eta], eta_ve, and per shear component the interpolated 1/eta and its eta_ve.
struct Pre {
    char* base = nullptr;
    long s1 = 0, s2 = 0, count = 0;  // element strides and elements per array
    int ne = 0;                      // shear components
    int own_ieta = 0;                // inv_eta computed here (the caller gave only eta)
};

template <class T>
DF<T> pre_view(const Pre& pr, int idx) {
    DF<T> v;
    v.p = reinterpret_cast<T*>(pr.base) + (long)idx * pr.count + 1 + pr.s1 + pr.s2;
    v.s1 = pr.s1;
    v.s2 = pr.s2;
    return v;
}

template <class T>
void apply_pre(SV<T>& v, const Pre* pr) {
    if (!pr || !pr->base) return;
    int idx = 0;
    if (pr->own_ieta) {
        v.ieta = pre_view<T>(*pr, idx++);
        v.has_ieta = 1;
    }
    v.eveC = pre_view<T>(*pr, idx++);
    for (int e = 0; e < pr->ne; ++e) {
        v.ievE[e] = pre_view<T>(*pr, idx++);
        v.eveE[e] = pre_view<T>(*pr, idx++);
    }
    v.has_pre = 1;
}

template <class T>
__global__ void inv_kernel(DF<T> dst, DF<T> src, int lo, int e0, int e1, int e2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + lo;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + lo;
    if (i > e0 || j > e1) return;
    for (int k = e2 < 0 ? 0 : lo; k <= (e2 < 0 ? 0 : e2); ++k) dst(i, j, k) = T(1) / src(i, j, k);
}

// Fill `pr` for the variable-viscosity field set `f` (scratch slot 2) and run the precompute.
template <class T, int ND>
int setup_pre(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, Pre* pr) {
    const long e0 = g->n[0] + 4, e1 = g->n[1] + 4, e2 = ND > 2 ? g->n[2] + 4 : 1;
    pr->s1 = e0;
    pr->s2 = ND > 2 ? e0 * e1 : 0;
    pr->count = e0 * e1 * e2;
    pr->ne = ND == 2 ? 1 : 3;
    pr->own_ieta = !cg_present(f->inv_eta);
    const int narr = pr->own_ieta + 1 + 2 * pr->ne;
    int rc = CG_OK;
    pr->base = static_cast<char*>(cg_scratch(ctx, 2, (size_t)narr * pr->count * sizeof(T), &rc));
    if (rc) return rc;
    SV<T> v = views<T>(f, ND);
    const dim3 block(32, 8);
    if (pr->own_ieta) {
        // 1/eta over the whole padded range the kernels read (logical -1 .. n+2)
        const DF<T> dst = pre_view<T>(*pr, 0);
        const dim3 gi(cg_div_up(g->n[0] + 4, 32), cg_div_up(g->n[1] + 4, 8));
        inv_kernel<T><<<gi, block, 0, ctx->stream>>>(dst, v.eta, -1, g->n[0] + 2, g->n[1] + 2, ND > 2 ? g->n[2] + 2 : -1);
        CG_CHECK_LAUNCH(ctx);
    }
    apply_pre(v, pr);
    precompute_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(v, scalars<T>(g, p), g->n[0] + 1,
                                                                                 g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// The weight fields of a FieldMask (cg_mask.at, indexed by location bits) as kernel views.
template <class T>
FieldMaskW<T> mask_views(const cg_mask* m) {
    FieldMaskW<T> w;
    std::memset(&w, 0, sizeof(w));
    for (int b = 0; b < 8; ++b)
        if (cg_present(m->at[b])) w.w[b] = cg_view<T>(m->at[b]);
    return w;
}

template <class T, int ND, class M>
void stress_launch(const cg_grid* g, const SV<T>& v, const SP<T>& s, bool res, const M& m, dim3 block, cudaStream_t st) {
    if (res)
        stress_kernel<T, ND, true, M><<<range_grid<ND>(g, block), block, 0, st>>>(v, s, g->n[0] + 1, g->n[1] + 1, m);
    else
        stress_kernel<T, ND, false, M><<<range_grid<ND>(g, block), block, 0, st>>>(v, s, g->n[0] + 1, g->n[1] + 1, m);
}

template <class T, int ND, class M>
void velocity_launch(const cg_grid* g, const SV<T>& v, const SP<T>& s, const BodyFn<T>& bf, bool res, const M& m,
                     dim3 block, cudaStream_t st) {
    if (res)
        velocity_kernel<T, ND, true, M><<<range_grid<ND>(g, block), block, 0, st>>>(v, s, bf, g->n[0] + 1, g->n[1] + 1, m);
    else
        velocity_kernel<T, ND, false, M><<<range_grid<ND>(g, block), block, 0, st>>>(v, s, bf, g->n[0] + 1, g->n[1] + 1, m);
}

// update_stress! over [0, n+1]^N; with `mask`, every strain-rate derivative is the masked
// operator ∂(V.d, ω, g, I) (src/GridOperators/masked_field_operators.jl:20-57).
template <class T, int ND>
cudaError_t stress_any(const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res, const Pre* pr,
                       const cg_mask* mask, dim3 block, cudaStream_t st) {
    SV<T> v = views<T>(f, ND);
    apply_pre(v, pr);
    const SP<T> s = scalars<T>(g, p);
    if (mask)
        stress_launch<T, ND>(g, v, s, res, mask_views<T>(mask), block, st);
    else
        stress_launch<T, ND>(g, v, s, res, NoMask<T>{}, block, st);
    return cudaGetLastError();
}

// update_velocity! over [0, n+1]^N; with `mask`, the pressure and stress derivatives are the
// masked operators.
template <class T, int ND>
cudaError_t velocity_any(const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res,
                         const Pre* pr, const cg_mask* mask, dim3 block, cudaStream_t st) {
    SV<T> v = views<T>(f, ND);
    apply_pre(v, pr);
    const SP<T> s = scalars<T>(g, p);
    if (mask)
        velocity_launch<T, ND>(g, v, s, body_fns<T>(g, p), res, mask_views<T>(mask), block, st);
    else
        velocity_launch<T, ND>(g, v, s, body_fns<T>(g, p), res, NoMask<T>{}, block, st);
    return cudaGetLastError();
}

template <class T, int ND>
int launch_stress(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res,
                  const Pre* pr = nullptr, const cg_mask* mask = nullptr, dim3 block = dim3(32, 8)) {
    const cudaError_t e = stress_any<T, ND>(g, f, p, res, pr, mask, block, ctx->stream);
    if (e != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "update_stress: %s", cudaGetErrorString(e));
    return CG_OK;
}

template <class T, int ND>
int launch_velocity(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res,
                    const Pre* pr = nullptr, const cg_mask* mask = nullptr, dim3 block = dim3(32, 8)) {
    const cudaError_t e = velocity_any<T, ND>(g, f, p, res, pr, mask, block, ctx->stream);
    if (e != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "update_velocity: %s", cudaGetErrorString(e));
    return CG_OK;
}

// Bytes from a field's first stored element to its last (the whole padded array).
size_t padded_span_bytes(const cg_field& f) {
    size_t span = 1;
    for (int d = 0; d < f.ndim; ++d) span += (size_t)(f.n[d] + 4 * f.halo[d] - 1) * (size_t)f.stride[d];
    return span * (f.dtype == CG_F64 ? 8 : 4);
}

// Block shapes of the stress and velocity kernels of a PT loop over this field set (tune_block;
// cached per grid, precision, layout and kernel form). The kernels update P, tau, V in place
// and write divV and r_V, so the candidates run on copies of those fields in a temporary
// allocation, released before the loop's graph is captured; the caller's fields are untouched.
template <class T, int ND>
int stokes_blocks(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, const Pre* pr,
                  const cg_mask* mask, dim3* bs, dim3* bv) {
    *bs = *bv = dim3(32, 8);
    dim3 forced;
    if (cg_block_forced(&forced)) {
        *bs = *bv = forced;
        return CG_OK;
    }
    if (!cg_autotune_enabled()) return CG_OK;
    std::string base = "stokes_blocks";
    cg_key_add(base, *g);
    cg_key_add(base, (int)sizeof(T));
    cg_key_add(base, f->V[0].stride);
    cg_key_add(base, f->tau[0].stride);
    cg_key_add(base, (int)cg_present(f->eta) + 2 * (int)cg_present(f->inv_eta) + 4 * (pr != nullptr) + 8 * (mask != nullptr));
    cg_key_add(base, ctx->num_sms);
    const std::string ks = base + "stress", kv = base + "velocity";
    cg_tune_cfg c1{0, 0}, c2{0, 0};
    if (cg_tune_lookup(ks, &c1) && cg_tune_lookup(kv, &c2)) {
        *bs = dim3((unsigned)c1.seg, (unsigned)c1.variant);
        *bv = dim3((unsigned)c2.seg, (unsigned)c2.variant);
        return CG_OK;
    }
    const int nt = ND == 2 ? 3 : 6;
    cg_stokes_fields c = *f;
    cg_field* upd[1 + 1 + 6 + 3 + 3];
    int nu = 0;
    upd[nu++] = &c.P;
    if (cg_present(c.divV)) upd[nu++] = &c.divV;
    for (int t = 0; t < nt; ++t) upd[nu++] = &c.tau[t];
    for (int d = 0; d < ND; ++d) {
        upd[nu++] = &c.V[d];
        if (cg_present(c.r_V[d])) upd[nu++] = &c.r_V[d];
    }
    size_t off[16], total = 0;
    for (int a = 0; a < nu; ++a) {
        off[a] = total;
        total += (padded_span_bytes(*upd[a]) + 255) & ~(size_t)255;
    }
    char* tmp = nullptr;
    if (cudaMalloc(&tmp, total) != cudaSuccess) {
        cudaGetLastError();
        return CG_OK;  // no room to time the candidates: the default shape
    }
    for (int a = 0; a < nu; ++a) {
        const cudaError_t e = cudaMemcpyAsync(tmp + off[a], upd[a]->data, padded_span_bytes(*upd[a]),
                                              cudaMemcpyDeviceToDevice, ctx->stream);
        if (e != cudaSuccess) {
            cudaFree(tmp);
            return cg_fail(ctx, CG_ERR_CUDA, "stokes block tuning: %s", cudaGetErrorString(e));
        }
        upd[a]->data = tmp + off[a];
    }
    *bs = cgk::tune_block("update_stress", ks,
                          [&](dim3 b) { return stress_any<T, ND>(g, &c, p, true, pr, mask, b, ctx->stream); }, ctx->stream);
    *bv = cgk::tune_block("update_velocity", kv,
                          [&](dim3 b) { return velocity_any<T, ND>(g, &c, p, true, pr, mask, b, ctx->stream); }, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(tmp);
    return CG_OK;
}

// The mask entries the masked Stokes kernels read, checked against the grid and dtype:
// update_stress! the velocity locations (bits 1 << d); update_velocity! the cell (0) and the
// shear locations (2D: 3; 3D: 3, 5, 6).
enum { MASK_STRESS = 1, MASK_VELOCITY = 2 };
int check_stokes_mask(cg_ctx* ctx, const cg_grid* g, const cg_mask* m, int dtype, int which) {
    if (!m) return cg_fail(ctx, CG_ERR_ARG, "masked stokes: mask is NULL");
    const int nd = g->ndim;
    int rc;
    if (which & MASK_STRESS)
        for (int d = 0; d < nd; ++d)
            if ((rc = cg_check_field(ctx, g, m->at[1 << d], dtype, 1 << d, "mask (velocity location)"))) return rc;
    if (which & MASK_VELOCITY) {
        if ((rc = cg_check_field(ctx, g, m->at[0], dtype, 0, "mask (cell)"))) return rc;
        const int shear[3] = {3, 5, 6};
        for (int e = 0; e < (nd == 2 ? 1 : 3); ++e)
            if ((rc = cg_check_field(ctx, g, m->at[shear[e]], dtype, shear[e], "mask (shear location)"))) return rc;
    }
    return CG_OK;
}

template <class T, int ND>
int launch_old(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f) {
    dim3 block(32, 8);
    update_old_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        views<T>(f, ND), cg_present(f->T) && cg_present(f->T_old), g->n[0] + 1, g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int launch_thermal_flux(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p) {
    dim3 block(32, 8);
    thermal_flux_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(views<T>(f, ND), scalars<T>(g, p),
                                                                                   g->n[0] + 1, g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int launch_thermal(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p) {
    dim3 block(32, 8);
    thermal_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(views<T>(f, ND), scalars<T>(g, p),
                                                                              g->n[0] + 1, g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// Fused thermal step Tin -> Tout (update_thermal_flux! + update_thermal!) over the launch range.
template <class T, int ND>
int launch_thermal_step(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                        const cg_field& Tin, const cg_field& Tout, cudaStream_t st) {
    ThermalStep<T> a;
    std::memset(&a, 0, sizeof(a));
    a.Tin = cg_view<T>(Tin);
    a.Told = cg_view<T>(f->T_old);
    a.Tout = cg_view<T>(Tout);
    for (int d = 0; d < ND; ++d) {
        a.V[d] = cg_view<T>(f->V[d]);
        a.idx[d] = (T)g->inv_spacing[d];
    }
    a.mlam = -(T)p->lambda_rhoCp;
    a.dt = (T)p->dt;
    dim3 block(32, 8);
    thermal_step_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, st>>>(a, g->n[0] + 1, g->n[1] + 1,
                                                                          ND > 2 ? g->n[2] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

#define SDISPATCH(fn, dtype, nd, ...)                                                              \
    ((dtype) == CG_F64 ? ((nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__))    \
                       : ((nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

// V boundary conditions of one PT iteration: bc!(V.d => bc_V[d]) as one batch.
int apply_bc_V(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_bc* bc_V) {
    if (!bc_V) return CG_OK;
    return cg_bc_apply_impl(ctx, g, g->ndim, f->V, bc_V);
}

// The library's partner buffer of T for the thermal ping-pong (scratch slot 0, T's layout).
int thermal_partner(cg_ctx* ctx, const cg_field& Tf, cg_field* out) {
    int rc = 0;
    void* p = cg_scratch(ctx, 0, padded_span_bytes(Tf), &rc);
    if (rc) return rc;
    *out = Tf;
    out->data = p;
    return CG_OK;
}

// `niter` PT iterations: update_stress!, update_velocity!, bc!(V) and, with bc_T, the thermal
// step and bc!(T) (examples/stokes_2d_inc_ve_T.jl:144-152). T alternates with the library's
// partner buffer and ends in f->T.
int pt_iterations(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                  const cg_bc* bc_V, int niter, int dtype, const Pre* pr = nullptr, const cg_bc* bc_T = nullptr,
                  const cg_mask* mask = nullptr) {
    cg_field Tw;
    std::memset(&Tw, 0, sizeof(Tw));
    if (bc_T) {
        int rc = thermal_partner(ctx, f->T, &Tw);
        if (rc) return rc;
    }
    std::string key = "stokes_pt";
    cg_key_add(key, *g);
    cg_key_add(key, *f);
    cg_key_add(key, *p);
    cg_key_add(key, niter);
    cg_bc none[3];
    std::memset(none, 0, sizeof(none));
    for (int d = 0; d < g->ndim; ++d) cg_key_add(key, bc_V ? bc_V[d] : none[d]);
    cg_key_add(key, pr ? pr->base : nullptr);
    cg_key_add(key, bc_T ? 1 : 0);
    if (bc_T) {
        cg_key_add(key, *bc_T);
        cg_key_add(key, Tw.data);
    }
    cg_key_add(key, mask ? 1 : 0);
    if (mask) cg_key_add(key, *mask);
    const int nd = g->ndim;
    dim3 bs, bv;
    int rc0 = SDISPATCH(stokes_blocks, dtype, nd, ctx, g, f, p, pr, mask, &bs, &bv);
    if (rc0) return rc0;
    cg_key_add(key, bs);
    cg_key_add(key, bv);
    const size_t tbytes = bc_T ? padded_span_bytes(f->T) : 0;
    return cg_graph_run(ctx, key, [&](cudaStream_t st) {
        // the partner starts as a copy, so that points no step writes agree in both buffers
        if (bc_T) CG_CUDA(ctx, cudaMemcpyAsync(Tw.data, f->T.data, tbytes, cudaMemcpyDeviceToDevice, st));
        for (int it = 0; it < niter; ++it) {
            const bool last = it == niter - 1;
            int rc = SDISPATCH(launch_stress, dtype, nd, ctx, g, f, p, last, pr, mask, bs);
            if (rc) return rc;
            rc = SDISPATCH(launch_velocity, dtype, nd, ctx, g, f, p, last, pr, mask, bv);
            if (rc) return rc;
            rc = apply_bc_V(ctx, g, f, bc_V);
            if (rc) return rc;
            if (bc_T) {
                const cg_field& src = (it % 2 == 0) ? f->T : Tw;
                const cg_field& dst = (it % 2 == 0) ? Tw : f->T;
                if ((rc = SDISPATCH(launch_thermal_step, dtype, nd, ctx, g, f, p, src, dst, st))) return rc;
                if ((rc = cg_bc_apply_impl(ctx, g, 1, &dst, bc_T))) return rc;
            }
        }
        if (bc_T && (niter & 1)) CG_CUDA(ctx, cudaMemcpyAsync(f->T.data, Tw.data, tbytes, cudaMemcpyDeviceToDevice, st));
        return (int)CG_OK;
    });
}

int residual(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, double tau_scale, double v_scale, double* err,
             int32_t* nonfinite) {
    const int nd = g->ndim;
    if (!cg_present(f->divV) || !cg_present(f->r_V[0]))
        return cg_fail(ctx, CG_ERR_ARG, "stokes residual: divV and r_V are required");
    // bc!(r_V.x => (x = Dirichlet(),), r_V.y => (y = Dirichlet(),), ...)
    cg_bc bcs[3];
    std::memset(bcs, 0, sizeof(bcs));
    for (int d = 0; d < nd; ++d) bcs[d].kind[d][0] = bcs[d].kind[d][1] = CG_BC_DIRICHLET;
    int rc = cg_bc_apply_impl(ctx, g, nd, f->r_V, bcs);
    if (rc) return rc;
    cg_field red[4];
    red[0] = f->divV;
    for (int d = 0; d < nd; ++d) red[1 + d] = f->r_V[d];
    if ((rc = cg_maxabs_enqueue(ctx, nd + 1, red))) return rc;
    double m[4];
    if ((rc = cg_maxabs_collect(ctx, nd + 1, red, m, nonfinite))) return rc;
    err[0] = m[0] * tau_scale;
    for (int d = 0; d < nd; ++d) err[1 + d] = m[1 + d] * v_scale;
    return CG_OK;
}

}  // namespace

extern "C" int cg_stokes_update_old(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_TAU | NEED_TAU_OLD, &dtype);
    if (rc) return rc;
    if (cg_present(f->T) != cg_present(f->T_old)) return cg_fail(ctx, CG_ERR_ARG, "update_old: T and T_old together");
    if (cg_present(f->T) && (rc = check_stokes(ctx, grid, f, NEED_TAU | NEED_T | NEED_TOLD, &dtype))) return rc;
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_old, dtype, grid->ndim, ctx, grid, f);
}

extern "C" int cg_stokes_update_stress(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                       const cg_stokes_params* p) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_stress: params is NULL");
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_stress, dtype, grid->ndim, ctx, grid, f, p, true);
}

extern "C" int cg_stokes_update_velocity(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                         const cg_stokes_params* p) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_velocity: params is NULL");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_velocity, dtype, grid->ndim, ctx, grid, f, p, true);
}

extern "C" int cg_stokes_update_thermal_flux(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                             const cg_stokes_params* p) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_T | NEED_QT, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_thermal_flux: params is NULL");
    if (f->V[0].dtype != dtype) return cg_fail(ctx, CG_ERR_ARG, "update_thermal_flux: V and T dtypes differ");
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_thermal_flux, dtype, grid->ndim, ctx, grid, f, p);
}

extern "C" int cg_stokes_update_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                        const cg_stokes_params* p) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_T | NEED_TOLD | NEED_QT, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_thermal: params is NULL");
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_thermal, dtype, grid->ndim, ctx, grid, f, p);
}

extern "C" int cg_stokes_pt_iterations(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                       const cg_stokes_params* p, const cg_bc* bc_V, int niter) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations: params is NULL");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    if (niter < 0) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations: niter < 0");
    if (niter == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    return pt_iterations(ctx, grid, f, p, bc_V, niter, dtype);
}

extern "C" int cg_stokes_update_stress_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                              const cg_stokes_params* p, const cg_mask* mask) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_stress_masked: params is NULL");
    if ((rc = check_stokes_mask(ctx, grid, mask, dtype, MASK_STRESS))) return rc;
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_stress, dtype, grid->ndim, ctx, grid, f, p, true, nullptr, mask);
}

extern "C" int cg_stokes_update_velocity_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                                const cg_stokes_params* p, const cg_mask* mask) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "update_velocity_masked: params is NULL");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    if ((rc = check_stokes_mask(ctx, grid, mask, dtype, MASK_VELOCITY))) return rc;
    cudaSetDevice(ctx->device);
    return SDISPATCH(launch_velocity, dtype, grid->ndim, ctx, grid, f, p, true, nullptr, mask);
}

extern "C" int cg_stokes_pt_iterations_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                              const cg_stokes_params* p, const cg_bc* bc_V, const cg_mask* mask,
                                              int niter) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_masked: params is NULL");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    if ((rc = check_stokes_mask(ctx, grid, mask, dtype, MASK_STRESS | MASK_VELOCITY))) return rc;
    if (niter < 0) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_masked: niter < 0");
    if (niter == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    return pt_iterations(ctx, grid, f, p, bc_V, niter, dtype, nullptr, nullptr, mask);
}

namespace {

template <class T>
Fused2D<T> fused_view(const cg_stokes_fields* in, const cg_stokes_fields* out, const cg_stokes_fields* a) {
    Fused2D<T> f;
    std::memset(&f, 0, sizeof(f));
    f.Vx_in = cg_view<T>(in->V[0]);
    f.Vy_in = cg_view<T>(in->V[1]);
    f.Vx_out = cg_view<T>(out->V[0]);
    f.Vy_out = cg_view<T>(out->V[1]);
    f.txx_in = cg_view<T>(in->tau[0]);
    f.tyy_in = cg_view<T>(in->tau[1]);
    f.txy_in = cg_view<T>(in->tau[2]);
    f.txx_out = cg_view<T>(out->tau[0]);
    f.tyy_out = cg_view<T>(out->tau[1]);
    f.txy_out = cg_view<T>(out->tau[2]);
    f.P_in = cg_view<T>(in->P);
    f.P_out = cg_view<T>(out->P);
    f.txx_o = cg_view<T>(a->tau_old[0]);
    f.tyy_o = cg_view<T>(a->tau_old[1]);
    f.txy_o = cg_view<T>(a->tau_old[2]);
    f.ieta = cg_view<T>(a->inv_eta);
    f.has_rho = cg_present(a->rho_g[0]) && cg_present(a->rho_g[1]);
    if (f.has_rho) {
        f.rhox = cg_view<T>(a->rho_g[0]);
        f.rhoy = cg_view<T>(a->rho_g[1]);
    }
    if (cg_present(a->divV)) f.divV = cg_view<T>(a->divV);
    if (cg_present(a->r_V[0])) {
        f.rVx = cg_view<T>(a->r_V[0]);
        f.rVy = cg_view<T>(a->r_V[1]);
    }
    return f;
}

template <class T>
Fused3D<T> fused3_view(const cg_stokes_fields* in, const cg_stokes_fields* out, const cg_stokes_fields* a) {
    Fused3D<T> f;
    std::memset(&f, 0, sizeof(f));
    for (int d = 0; d < 3; ++d) {
        f.V_in[d] = cg_view<T>(in->V[d]);
        f.V_out[d] = cg_view<T>(out->V[d]);
        f.has_rho[d] = cg_present(a->rho_g[d]);
        if (f.has_rho[d]) f.rho[d] = cg_view<T>(a->rho_g[d]);
        if (cg_present(a->r_V[d])) f.rV[d] = cg_view<T>(a->r_V[d]);
    }
    for (int c = 0; c < 6; ++c) {
        f.tau_in[c] = cg_view<T>(in->tau[c]);
        f.tau_out[c] = cg_view<T>(out->tau[c]);
        f.tau_o[c] = cg_view<T>(a->tau_old[c]);
    }
    f.P_in = cg_view<T>(in->P);
    f.P_out = cg_view<T>(out->P);
    f.ieta = cg_view<T>(a->inv_eta);
    if (cg_present(a->divV)) f.divV = cg_view<T>(a->divV);
    return f;
}

template <class T>
int pp_iterations_3d(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* a, const cg_stokes_fields* b,
                     const cg_stokes_params* p, const cg_bc* bc_V, int niter) {
    const Fused3D<T> fab = fused3_view<T>(a, b, a), fba = fused3_view<T>(b, a, a);
    const SP<T> s = scalars<T>(g, p);
    const bool res = cg_present(a->divV) && cg_present(a->r_V[0]);
    // tensor maps of the TMA-fed variants (FP32 layouts that allow them)
    m3t::Tma tma;
    int* err = nullptr;
    if constexpr (sizeof(T) == 4) {
        int rc = CG_OK;
        err = cg_tma_flag(ctx, &rc);
        if (rc) return rc;
        const cg_field* Va[3] = {&a->V[0], &a->V[1], &a->V[2]};
        const cg_field* Vb[3] = {&b->V[0], &b->V[1], &b->V[2]};
        const cg_field *ta[6], *tb[6], *to[6];
        for (int c = 0; c < 6; ++c) {
            ta[c] = &a->tau[c];
            tb[c] = &b->tau[c];
            to[c] = &a->tau_old[c];
        }
        const cg_field* rho[3] = {&a->rho_g[0], &a->rho_g[1], &a->rho_g[2]};
        tma = m3t::make_tma(Va, &a->P, ta, Vb, &b->P, tb, &a->inv_eta, to, nullptr, rho, g->n, err);
    }
    const M3Launch lab = m3_launch_of(&tma, true), lba = m3_launch_of(&tma, false);
    const cg_tune_cfg tc = tune_march3d(fab, s, g->n[0], g->n[1], g->n[2], ctx->num_sms, ctx->stream, lab);
    const bool staged = tma.ok && tc.variant >= kM3TmaFirst;
    std::string key = "stokes_pp3";
    cg_key_add(key, tc);
    if (staged) cg_key_add(key, cg_tma_wait_cfg());
    cg_key_add(key, *g);
    cg_key_add(key, *a);
    cg_key_add(key, *b);
    cg_key_add(key, *p);
    cg_key_add(key, niter);
    cg_bc none[3];
    std::memset(none, 0, sizeof(none));
    for (int d = 0; d < 3; ++d) cg_key_add(key, bc_V ? bc_V[d] : none[d]);
    const int rc = cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int it = 0; it < niter; ++it) {
            const Fused3D<T>& fk = (it % 2 == 0) ? fab : fba;
            const M3Launch& lk = (it % 2 == 0) ? lab : lba;
            const int nsm = ctx->num_sms;
            const cudaError_t le =
                (res && it == niter - 1)
                    ? launch_march3d_any<T, true>(fk, s, g->n[0], g->n[1], g->n[2], nsm, tc.seg, st, tc.variant, it > 0, lk)
                    : launch_march3d_any<T, false>(fk, s, g->n[0], g->n[1], g->n[2], nsm, tc.seg, st, tc.variant, it > 0, lk);
            if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused3d launch: %s", cudaGetErrorString(le));
            if (bc_V) {
                // no dependent launches around the TMA-fed kernel (measured slower with them)
                int r = cg_bc_apply_impl(ctx, g, 3, (it % 2 == 0) ? b->V : a->V, bc_V, !staged);
                if (r) return r;
            }
        }
        return (int)CG_OK;
    });
    if (rc || !staged) return rc;
    return cg_tma_check(ctx, err, "fused3d iteration");
}

template <class T>
int pp_iterations_t(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* a, const cg_stokes_fields* b,
                    const cg_stokes_params* p, const cg_bc* bc_V, int niter) {
    if (g->ndim == 3) return pp_iterations_3d<T>(ctx, g, a, b, p, bc_V, niter);
    Fused2D<T> fab = fused_view<T>(a, b, a), fba = fused_view<T>(b, a, a);
    // from the second iteration on, bc!(V) of the previous one is folded into the velocity
    // reads; one launch at the end patches the outputs of the last two iterations
    const Fused2D<T> fab0 = fab;
    VFold<T> vf;
    const bool fold = cg_bc_fold_enabled() && make_vfold(g, bc_V, &vf);
    if (fold) fab.bc = fba.bc = vf;
    const SP<T> s = scalars<T>(g, p);
    const bool res = cg_present(a->divV) && cg_present(a->r_V[0]);
    const cg_tune_cfg tc = tune_march2d(fab, s, g->n[0], g->n[1], ctx->num_sms, ctx->stream);
    std::string key = "stokes_pp";
    cg_key_add(key, tc);
    cg_key_add(key, *g);
    cg_key_add(key, *a);
    cg_key_add(key, *b);
    cg_key_add(key, *p);
    cg_key_add(key, niter);
    cg_bc none[2];
    std::memset(none, 0, sizeof(none));
    for (int d = 0; d < 2; ++d) cg_key_add(key, bc_V ? bc_V[d] : none[d]);
    cg_key_add(key, (int)fold);
    // two iterations per pass (the tuner's variant 1) where no bc!(V) launch is needed between
    // iterations: an even number of passes (a -> b, b -> a) leaves at least the last two
    // iterations to the one-iteration kernel, so that a ends with the state after niter
    // iterations and b with the state after niter - 1, as in the one-iteration form
    const bool x2 = tc.variant >= 1 && (fold || !bc_V);
    const int npass = x2 ? ((niter / 2 - 1) & ~1) : 0;
    return cg_graph_run(ctx, key, [&](cudaStream_t st) {
        for (int k = 0; k < npass; ++k) {
            const Fused2D<T>& fk = (k % 2 == 0) ? fab : fba;
            const int nsm = ctx->num_sms;
            const bool last = 2 * k + 2 == niter;
            const cudaError_t le = (res && last)
                                       ? launch_march2d_x2<T, true>(fk, s, g->n[0], g->n[1], nsm, tc.seg, k > 0, st, k > 0, tc.variant)
                                       : launch_march2d_x2<T, false>(fk, s, g->n[0], g->n[1], nsm, tc.seg, k > 0, st, k > 0, tc.variant);
            if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused2d x2 launch: %s", cudaGetErrorString(le));
        }
        for (int it = 2 * npass; it < niter; ++it) {
            const Fused2D<T>& fk = it == 0 ? fab0 : (it % 2 == 0) ? fab : fba;
            const int nsm = ctx->num_sms;
            const cudaError_t le = (res && it == niter - 1)
                                       ? launch_march2d<T, true>(fk, s, g->n[0], g->n[1], nsm, tc.seg, st, it > 0)
                                       : launch_march2d<T, false>(fk, s, g->n[0], g->n[1], nsm, tc.seg, st, it > 0);
            if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused2d launch: %s", cudaGetErrorString(le));
            if (bc_V && !fold) {
                int r = cg_bc_apply_impl(ctx, g, 2, (it % 2 == 0) ? b->V : a->V, bc_V, true);
                if (r) return r;
            }
        }
        if (fold) {
            const cg_field fl[4] = {b->V[0], b->V[1], a->V[0], a->V[1]};
            const cg_bc bl[4] = {bc_V[0], bc_V[1], bc_V[0], bc_V[1]};
            int r = cg_bc_apply_impl(ctx, g, niter > 1 ? 4 : 2, fl, bl, true);
            if (r) return r;
        }
        return (int)CG_OK;
    });
}

}  // namespace

extern "C" int cg_stokes_pt_iterations_pp(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* a,
                                          const cg_stokes_fields* b, const cg_stokes_params* p, const cg_bc* bc_V,
                                          int niter) {
    int dtype;
    int rc = check_stokes(ctx, grid, a, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!b || !p) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_pp: NULL argument");
    for (int d = 0; d < 3; ++d)
        if (p->rho_g_fn[d].kind != CG_FN_NONE)
            return cg_fail(ctx, CG_ERR_UNSUPPORTED, "pt_iterations_pp: body forces are read from arrays (rho_g_fn[%d] set)", d);
    if (grid->ndim < 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "pt_iterations_pp: 2D and 3D grids only");
    if (!cg_present(a->inv_eta)) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_pp: inv_eta is required");
    if (niter < 0 || (niter & 1)) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_pp: niter must be even and >= 0");
    int dtb;
    if ((rc = check_stokes(ctx, grid, b, NEED_V | NEED_TAU | NEED_P, &dtb))) return rc;
    if (dtb != dtype) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_pp: a and b dtypes differ");
    if (cg_present(a->divV) != cg_present(a->r_V[0]))
        return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_pp: divV and r_V together");
    if (niter == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    return dtype == CG_F64 ? pp_iterations_t<double>(ctx, grid, a, b, p, bc_V, niter)
                           : pp_iterations_t<float>(ctx, grid, a, b, p, bc_V, niter);
}

extern "C" int cg_stokes_residual(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, double tau_scale,
                                  double v_scale, double* err_host) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_P, &dtype);
    if (rc) return rc;
    if (!err_host) return cg_fail(ctx, CG_ERR_ARG, "stokes_residual: err is NULL");
    cudaSetDevice(ctx->device);
    int32_t bad = 0;
    rc = residual(ctx, grid, f, tau_scale, v_scale, err_host, &bad);
    if (rc) return rc;
    return bad ? cg_fail(ctx, CG_ERR_NONFINITE, "stokes_residual: non-finite residual") : CG_OK;
}

namespace {

int check_solve(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                const cg_solve_opts* o, cg_solve_result* res, int* dtype) {
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, dtype);
    if (rc) return rc;
    if (!p || !o || !res) return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: NULL argument");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    if (o->ncheck < 1 || o->max_iter < 1) return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: ncheck/max_iter < 1");
    if (!cg_present(f->divV) || !cg_present(f->r_V[0]))
        return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: divV and r_V are required for the convergence check");
    if (*dtype != CG_F64) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve: the solution fields must be FP64");
    if (o->precision != CG_F64 && o->precision != CG_F32)
        return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: precision must be CG_F64 or CG_F32");
    return CG_OK;
}

// The reference PT loop in FP64 (examples/stokes_2d_inc_ve_T.jl:144-163): graph-replayed
// chunks of ncheck iterations, then the convergence measures. With bc_T, every iteration also
// takes the thermal step.
int solve_fp64(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
               const cg_bc* bc_V, const cg_bc* bc_T, const cg_solve_opts* o, cg_solve_result* res, int dtype) {
    int rc;
    // variable viscosity: precompute the viscosity terms once for the whole solve
    Pre pre;
    const bool var = cg_present(f->eta) || cg_present(f->inv_eta);
    if (var && (rc = SDISPATCH(setup_pre, dtype, grid->ndim, ctx, grid, f, p, &pre))) return rc;
    std::memset(res, 0, sizeof(*res));
    CG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    int iter = 0;
    int status = CG_ERR_NOCONV;
    while (iter < o->max_iter) {
        const int chunk = std::min(o->ncheck, o->max_iter - iter);
        if ((rc = pt_iterations(ctx, grid, f, p, bc_V, chunk, dtype, var ? &pre : nullptr, bc_T))) return rc;
        iter += chunk;
        if (chunk < o->ncheck) break;  // the reference only checks at multiples of ncheck
        int32_t bad = 0;
        if ((rc = residual(ctx, grid, f, o->tau_scale, o->v_scale, res->err, &bad))) return rc;
        res->checks++;
        if (bad) {
            status = CG_ERR_NONFINITE;
            cg_fail(ctx, CG_ERR_NONFINITE, "stokes_solve: non-finite residual after %d iterations", iter);
            break;
        }
        bool conv = true;
        for (int c = 0; c <= grid->ndim; ++c) conv = conv && res->err[c] < o->eps;
        if (conv) {
            status = CG_OK;
            res->converged = 1;
            break;
        }
    }
    CG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    CG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->seconds = ms * 1e-3;
    res->iterations = iter;
    if (status == CG_ERR_NOCONV) cg_fail(ctx, CG_ERR_NOCONV, "stokes_solve: not converged after %d iterations", iter);
    return status;
}

int check_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, int dtype) {
    int rc;
    if ((rc = cg_check_field(ctx, grid, f->T, dtype, 0, "T"))) return rc;
    if ((rc = cg_check_field(ctx, grid, f->T_old, dtype, 0, "T_old"))) return rc;
    return CG_OK;
}

}  // namespace

extern "C" int cg_stokes_solve(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                               const cg_bc* bc_V, const cg_solve_opts* o, cg_solve_result* res) {
    int dtype;
    int rc = check_solve(ctx, grid, f, p, o, res, &dtype);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    if (o->precision == CG_F32) return cg_stokes_solve_dc(ctx, grid, f, p, bc_V, o, res);
    return solve_fp64(ctx, grid, f, p, bc_V, nullptr, o, res, dtype);
}

extern "C" int cg_stokes_solve_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                       const cg_stokes_params* p, const cg_bc* bc_V, const cg_bc* bc_T,
                                       const cg_solve_opts* o, cg_solve_result* res) {
    int dtype;
    int rc = check_solve(ctx, grid, f, p, o, res, &dtype);
    if (rc) return rc;
    if (!bc_T) return cg_fail(ctx, CG_ERR_ARG, "stokes_solve_thermal: bc_T is NULL");
    if ((rc = check_thermal(ctx, grid, f, dtype))) return rc;
    if (o->precision != CG_F64)
        return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve_thermal: FP64 PT only (precision CG_F64)");
    cudaSetDevice(ctx->device);
    return solve_fp64(ctx, grid, f, p, bc_V, bc_T, o, res, dtype);
}

extern "C" int cg_stokes_pt_iterations_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                               const cg_stokes_params* p, const cg_bc* bc_V, const cg_bc* bc_T,
                                               int niter) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p || !bc_T) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_thermal: NULL argument");
    if ((rc = check_body(ctx, grid, f, p))) return rc;
    if ((rc = check_thermal(ctx, grid, f, dtype))) return rc;
    if (niter < 0) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations_thermal: niter < 0");
    if (niter == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    return pt_iterations(ctx, grid, f, p, bc_V, niter, dtype, nullptr, bc_T);
}

extern "C" int cg_stokes_thermal_step(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                      const cg_stokes_params* p, const cg_bc* bc_T, const cg_field* T_out) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V, &dtype);
    if (rc) return rc;
    if (!p || !T_out) return cg_fail(ctx, CG_ERR_ARG, "thermal_step: NULL argument");
    if ((rc = check_thermal(ctx, grid, f, dtype))) return rc;
    if ((rc = cg_check_field(ctx, grid, *T_out, dtype, 0, "T_out"))) return rc;
    if (T_out->data == f->T.data) return cg_fail(ctx, CG_ERR_ARG, "thermal_step: T_out must not be T");
    cudaSetDevice(ctx->device);
    if ((rc = SDISPATCH(launch_thermal_step, dtype, grid->ndim, ctx, grid, f, p, f->T, *T_out, ctx->stream))) return rc;
    return bc_T ? cg_bc_apply_impl(ctx, grid, 1, T_out, bc_T) : CG_OK;
}
