// cg_stokes.cu — pseudo-transient viscoelastic Stokes kernels
// (Chmy.jl examples/stokes_2d_inc_ve_T.jl:11-60, examples/stokes_3d_inc_ve_T.jl:11-77).
#include "cg_common.cuh"

int cg_bc_apply_impl(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs);
int cg_maxabs_enqueue(cg_ctx* ctx, int nfields, const cg_field* fields);
int cg_maxabs_collect(cg_ctx* ctx, int nfields, const cg_field* fields, double* out, int32_t* nonfinite);

namespace {

template <class T>
struct SV {  // device views of the Stokes field set
    DF<T> V[3], rV[3], P, divV, tau[6], tau_old[6], eta, ieta, rho[3], Tt, To, qT[3];
    int has_rV, has_divV, has_eta, has_ieta, has_rho[3];
    // 1/eta at a cell: the precomputed field when given, else an IEEE division (same bits)
    __device__ __forceinline__ T inv_eta(int i, int j, int k) const {
        return has_ieta ? ieta(i, j, k) : T(1) / eta(i, j, k);
    }
};

template <class T>
struct SP {  // scalars in the field precision
    T eta, eta_ve, G, dt, dtau_Pr, dtau_r, nu_dtau, lam;
    T inv_Gdt, third;
    T idx[3];
};

template <class T>
SV<T> views(const cg_stokes_fields* f, int nd) {
    SV<T> v;
    std::memset(&v, 0, sizeof(v));
    const int nt = nd == 2 ? 3 : 6;
    for (int d = 0; d < nd; ++d) {
        v.V[d] = cg_view<T>(f->V[d]);
        if (cg_present(f->r_V[d])) v.rV[d] = cg_view<T>(f->r_V[d]);
        if (cg_present(f->rho_g[d])) {
            v.rho[d] = cg_view<T>(f->rho_g[d]);
            v.has_rho[d] = 1;
        }
        if (cg_present(f->qT[d])) v.qT[d] = cg_view<T>(f->qT[d]);
    }
    v.has_rV = cg_present(f->r_V[0]);
    for (int c = 0; c < nt; ++c) {
        v.tau[c] = cg_view<T>(f->tau[c]);
        if (cg_present(f->tau_old[c])) v.tau_old[c] = cg_view<T>(f->tau_old[c]);
    }
    v.P = cg_view<T>(f->P);
    if (cg_present(f->divV)) {
        v.divV = cg_view<T>(f->divV);
        v.has_divV = 1;
    }
    if (cg_present(f->eta)) {
        v.eta = cg_view<T>(f->eta);
        v.has_eta = 1;
    }
    if (cg_present(f->inv_eta)) {
        v.ieta = cg_view<T>(f->inv_eta);
        v.has_ieta = 1;
        v.has_eta = 1;
    }
    if (cg_present(f->T)) v.Tt = cg_view<T>(f->T);
    if (cg_present(f->T_old)) v.To = cg_view<T>(f->T_old);
    return v;
}

template <class T>
SP<T> scalars(const cg_grid* g, const cg_stokes_params* p) {
    SP<T> s;
    s.eta = (T)p->eta;
    s.eta_ve = (T)p->eta_ve;
    s.G = (T)p->G;
    s.dt = (T)p->dt;
    s.dtau_Pr = (T)p->dtau_Pr;
    s.dtau_r = (T)p->dtau_r;
    s.nu_dtau = (T)p->nu_dtau;
    s.lam = (T)p->lambda_rhoCp;
    s.inv_Gdt = T(1) / (s.G * s.dt);
    s.third = T(1) / T(3);
    for (int d = 0; d < 3; ++d) s.idx[d] = (T)g->inv_spacing[d];
    return s;
}

template <class T>
__device__ __forceinline__ T eta_ve_of(T eta, T G, T dt) {
    return T(1.0) / (T(1.0) / eta + T(1.0) / (G * dt));
}

// 2D/3D launch: x, y threads over [0, n+1]; z over blockIdx.z.
template <int ND>
inline dim3 range_grid(const cg_grid* g, dim3 block) {
    return dim3(cg_div_up(g->n[0] + 2, block.x), cg_div_up(g->n[1] + 2, block.y), ND > 2 ? g->n[2] + 2 : 1);
}

// update_stress! at one point. Tensor order 2D (xx, yy, xy), 3D (xx, yy, zz, xy, xz, yz).
template <class T, int ND, bool WRITE_RES>
__global__ void stress_kernel(const SV<T> v, const SP<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const DF<T>& Vx = v.V[0];
    const DF<T>& Vy = v.V[1];
    // ∂x(V.x) at Center: V.x is Vertex in x -> V.x[i+1] - V.x[i]
    const T exx = (Vx(i + 1, j, k) - Vx(i, j, k)) * s.idx[0];
    const T eyy = (Vy(i, j + 1, k) - Vy(i, j, k)) * s.idx[1];
    T dv = exx + eyy;
    T ezz = T(0);
    if (ND > 2) {
        const DF<T>& Vz = v.V[2];
        ezz = (Vz(i, j, k + 1) - Vz(i, j, k)) * s.idx[2];
        dv = dv + ezz;
    }
    if (WRITE_RES && v.has_divV) v.divV(i, j, k) = dv;
    T ieta_c = T(0), eve_c = s.eta_ve;
    if (v.has_eta) {
        ieta_c = v.inv_eta(i, j, k);
        eve_c = T(1) / (ieta_c + s.inv_Gdt);
    }
    v.P(i, j, k) = v.P(i, j, k) - dv * eve_c * s.dtau_Pr;
    auto diag = [&](int c, T edd) {
        const T t = v.tau[c](i, j, k), to = v.tau_old[c](i, j, k);
        T r;
        if (v.has_eta)
            r = -(t - to) * s.inv_Gdt - t * ieta_c + T(2.0) * (edd - dv * s.third);
        else  // examples/stokes_2d_inc_ve_T.jl:28-29, literally
            r = -(t - to) / (s.G * s.dt) - t / s.eta + T(2.0) * (edd - dv / T(3.0));
        v.tau[c](i, j, k) = t + r * eve_c * s.dtau_r;
    };
    // shear component on the (a, b) edge: 1/eta interpolated with the Linear rule over the 4
    // cells around it, dim a innermost (interpolation.jl:217-221) = harmonic mean of eta
    auto shear = [&](int c, T eod, int a, int b) {
        const T t = v.tau[c](i, j, k), to = v.tau_old[c](i, j, k);
        if (v.has_eta) {
            const int ai = a == 0, aj = a == 1, ak = a == 2;
            const int bi = b == 0, bj = b == 1, bk = b == 2;
            const T e00 = v.inv_eta(i - ai - bi, j - aj - bj, k - ak - bk);
            const T e10 = v.inv_eta(i - bi, j - bj, k - bk);
            const T e01 = v.inv_eta(i - ai, j - aj, k - ak);
            const T e11 = v.inv_eta(i, j, k);
            const T lo = fma(T(0.5), e10 - e00, e00);
            const T hi = fma(T(0.5), e11 - e01, e01);
            const T iev = fma(T(0.5), hi - lo, lo);
            const T eve = T(1) / (iev + s.inv_Gdt);
            const T r = -(t - to) * s.inv_Gdt - t * iev + T(2.0) * eod;
            v.tau[c](i, j, k) = t + r * eve * s.dtau_r;
        } else {  // examples/stokes_2d_inc_ve_T.jl:30
            const T r = -(t - to) / (s.G * s.dt) - t / s.eta + T(2.0) * eod;
            v.tau[c](i, j, k) = t + r * s.eta_ve * s.dtau_r;
        }
    };
    // ∂y(V.x) at the xy vertex: V.x is Center in y -> V.x[j] - V.x[j-1]
    const T exy = T(0.5) * ((Vx(i, j, k) - Vx(i, j - 1, k)) * s.idx[1] + (Vy(i, j, k) - Vy(i - 1, j, k)) * s.idx[0]);
    if (ND == 2) {
        diag(0, exx);
        diag(1, eyy);
        shear(2, exy, 0, 1);
    } else {
        const DF<T>& Vz = v.V[2];
        const T exz = T(0.5) * ((Vx(i, j, k) - Vx(i, j, k - 1)) * s.idx[2] + (Vz(i, j, k) - Vz(i - 1, j, k)) * s.idx[0]);
        const T eyz = T(0.5) * ((Vy(i, j, k) - Vy(i, j, k - 1)) * s.idx[2] + (Vz(i, j, k) - Vz(i, j - 1, k)) * s.idx[1]);
        diag(0, exx);
        diag(1, eyy);
        diag(2, ezz);
        shear(3, exy, 0, 1);
        shear(4, exz, 0, 2);
        shear(5, eyz, 1, 2);
    }
}

// update_velocity! at one point.
template <class T, int ND, bool WRITE_RES>
__global__ void velocity_kernel(const SV<T> v, const SP<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const DF<T>& P = v.P;
    // tensor components: 2D xx=0 yy=1 xy=2; 3D xx=0 yy=1 zz=2 xy=3 xz=4 yz=5
    const int XY = ND == 2 ? 2 : 3;
    const DF<T>& txx = v.tau[0];
    const DF<T>& tyy = v.tau[1];
    const DF<T>& txy = v.tau[XY];
    // P, τ_dd are Center: at a face along d, left = I - e_d, right = I.
    // τ_xy is Vertex in x and y: ∂y(τxy) at a V.x face (Vertex x, Center y) -> τxy[j+1] - τxy[j].
    T rx = -((P(i, j, k) - P(i - 1, j, k)) * s.idx[0]) + (txx(i, j, k) - txx(i - 1, j, k)) * s.idx[0];
    rx = rx + (txy(i, j + 1, k) - txy(i, j, k)) * s.idx[1];
    T ry = -((P(i, j, k) - P(i, j - 1, k)) * s.idx[1]) + (tyy(i, j, k) - tyy(i, j - 1, k)) * s.idx[1];
    ry = ry + (txy(i + 1, j, k) - txy(i, j, k)) * s.idx[0];
    T rz = T(0);
    if (ND > 2) {
        const DF<T>& tzz = v.tau[2];
        const DF<T>& txz = v.tau[4];
        const DF<T>& tyz = v.tau[5];
        rx = rx + (txz(i, j, k + 1) - txz(i, j, k)) * s.idx[2];
        ry = ry + (tyz(i, j, k + 1) - tyz(i, j, k)) * s.idx[2];
        rz = -((P(i, j, k) - P(i, j, k - 1)) * s.idx[2]) + (tzz(i, j, k) - tzz(i, j, k - 1)) * s.idx[2];
        rz = rz + (txz(i + 1, j, k) - txz(i, j, k)) * s.idx[0];
        rz = rz + (tyz(i, j + 1, k) - tyz(i, j, k)) * s.idx[1];
    }
    if (v.has_rho[0]) rx = rx - v.rho[0](i, j, k);
    if (v.has_rho[1]) ry = ry - v.rho[1](i, j, k);
    if (ND > 2 && v.has_rho[2]) rz = rz - v.rho[2](i, j, k);
    if (WRITE_RES && v.has_rV) {
        v.rV[0](i, j, k) = rx;
        v.rV[1](i, j, k) = ry;
        if (ND > 2) v.rV[2](i, j, k) = rz;
    }
    if (v.has_eta) {
        // nu_dtau / max(eta_ve) of the two cells beside the face, without a division
        const T c = v.inv_eta(i, j, k);
        v.V[0](i, j, k) = v.V[0](i, j, k) + rx * (s.nu_dtau * (fmin(v.inv_eta(i - 1, j, k), c) + s.inv_Gdt));
        v.V[1](i, j, k) = v.V[1](i, j, k) + ry * (s.nu_dtau * (fmin(v.inv_eta(i, j - 1, k), c) + s.inv_Gdt));
        if (ND > 2)
            v.V[2](i, j, k) = v.V[2](i, j, k) + rz * (s.nu_dtau * (fmin(v.inv_eta(i, j, k - 1), c) + s.inv_Gdt));
    } else {  // examples/stokes_2d_inc_ve_T.jl:41-42
        v.V[0](i, j, k) = v.V[0](i, j, k) + rx * s.nu_dtau / s.eta_ve;
        v.V[1](i, j, k) = v.V[1](i, j, k) + ry * s.nu_dtau / s.eta_ve;
        if (ND > 2) v.V[2](i, j, k) = v.V[2](i, j, k) + rz * s.nu_dtau / s.eta_ve;
    }
}

template <class T, int ND>
__global__ void update_old_kernel(const SV<T> v, int has_T, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    if (has_T) v.To(i, j, k) = v.Tt(i, j, k);
#pragma unroll
    for (int c = 0; c < (ND == 2 ? 3 : 6); ++c) v.tau_old[c](i, j, k) = v.tau[c](i, j, k);
}

template <class T, int ND>
__global__ void thermal_flux_kernel(const SV<T> v, const SP<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const DF<T>& Tt = v.Tt;
    const T c = Tt(i, j, k);
    const T mlam = -s.lam;
    {
        const T l = Tt(i - 1, j, k), vv = v.V[0](i, j, k);
        v.qT[0](i, j, k) = mlam * ((c - l) * s.idx[0]) + fmax(vv, T(0.0)) * l + fmin(vv, T(0.0)) * c;
    }
    {
        const T l = Tt(i, j - 1, k), vv = v.V[1](i, j, k);
        v.qT[1](i, j, k) = mlam * ((c - l) * s.idx[1]) + fmax(vv, T(0.0)) * l + fmin(vv, T(0.0)) * c;
    }
    if (ND > 2) {
        const T l = Tt(i, j, k - 1), vv = v.V[2](i, j, k);
        v.qT[2](i, j, k) = mlam * ((c - l) * s.idx[2]) + fmax(vv, T(0.0)) * l + fmin(vv, T(0.0)) * c;
    }
}

template <class T, int ND>
__global__ void thermal_kernel(const SV<T> v, const SP<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    T dv = (v.qT[0](i + 1, j, k) - v.qT[0](i, j, k)) * s.idx[0];
    dv = dv + (v.qT[1](i, j + 1, k) - v.qT[1](i, j, k)) * s.idx[1];
    if (ND > 2) dv = dv + (v.qT[2](i, j, k + 1) - v.qT[2](i, j, k)) * s.idx[2];
    v.Tt(i, j, k) = v.To(i, j, k) - s.dt * dv;
}

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

template <class T, int ND>
int launch_stress(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res) {
    dim3 block(32, 8);
    const SV<T> v = views<T>(f, ND);
    const SP<T> s = scalars<T>(g, p);
    if (res)
        stress_kernel<T, ND, true><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(v, s, g->n[0] + 1, g->n[1] + 1);
    else
        stress_kernel<T, ND, false><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(v, s, g->n[0] + 1, g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int launch_velocity(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p, bool res) {
    dim3 block(32, 8);
    const SV<T> v = views<T>(f, ND);
    const SP<T> s = scalars<T>(g, p);
    if (res)
        velocity_kernel<T, ND, true><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(v, s, g->n[0] + 1, g->n[1] + 1);
    else
        velocity_kernel<T, ND, false><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(v, s, g->n[0] + 1, g->n[1] + 1);
    CG_CHECK_LAUNCH(ctx);
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

#define SDISPATCH(fn, dtype, nd, ...)                                                              \
    ((dtype) == CG_F64 ? ((nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__))    \
                       : ((nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

// V boundary conditions of one PT iteration: bc!(V.d => bc_V[d]) as one batch.
int apply_bc_V(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_bc* bc_V) {
    if (!bc_V) return CG_OK;
    return cg_bc_apply_impl(ctx, g, g->ndim, f->V, bc_V);
}

int pt_iterations(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                  const cg_bc* bc_V, int niter, int dtype) {
    std::string key = "stokes_pt";
    cg_key_add(key, *g);
    cg_key_add(key, *f);
    cg_key_add(key, *p);
    cg_key_add(key, niter);
    cg_bc none[3];
    std::memset(none, 0, sizeof(none));
    for (int d = 0; d < g->ndim; ++d) cg_key_add(key, bc_V ? bc_V[d] : none[d]);
    const int nd = g->ndim;
    return cg_graph_run(ctx, key, [&](cudaStream_t) {
        for (int it = 0; it < niter; ++it) {
            const bool last = it == niter - 1;
            int rc = SDISPATCH(launch_stress, dtype, nd, ctx, g, f, p, last);
            if (rc) return rc;
            rc = SDISPATCH(launch_velocity, dtype, nd, ctx, g, f, p, last);
            if (rc) return rc;
            rc = apply_bc_V(ctx, g, f, bc_V);
            if (rc) return rc;
        }
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
    if (niter < 0) return cg_fail(ctx, CG_ERR_ARG, "pt_iterations: niter < 0");
    if (niter == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    return pt_iterations(ctx, grid, f, p, bc_V, niter, dtype);
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

extern "C" int cg_stokes_solve(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                               const cg_bc* bc_V, const cg_solve_opts* o, cg_solve_result* res) {
    int dtype;
    int rc = check_stokes(ctx, grid, f, NEED_V | NEED_TAU | NEED_TAU_OLD | NEED_P, &dtype);
    if (rc) return rc;
    if (!p || !o || !res) return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: NULL argument");
    if (o->ncheck < 1 || o->max_iter < 1) return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: ncheck/max_iter < 1");
    if (!cg_present(f->divV) || !cg_present(f->r_V[0]))
        return cg_fail(ctx, CG_ERR_ARG, "stokes_solve: divV and r_V are required for the convergence check");
    if (o->precision != CG_F64 || dtype != CG_F64)
        return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve: FP64 fields and precision only in this call");
    cudaSetDevice(ctx->device);
    std::memset(res, 0, sizeof(*res));
    CG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    int iter = 0;
    int status = CG_ERR_NOCONV;
    while (iter < o->max_iter) {
        const int chunk = std::min(o->ncheck, o->max_iter - iter);
        if ((rc = pt_iterations(ctx, grid, f, p, bc_V, chunk, dtype))) return rc;
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
