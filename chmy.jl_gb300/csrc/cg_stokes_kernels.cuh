// cg_stokes_kernels.cuh — device code of the VE Stokes PT kernels shared by the per-kernel
// entry points (cg_stokes.cu) and the defect-correction solver (cg_stokes_dc.cu).
#pragma once

#include "cg_common.cuh"

namespace cgk {


template <class T>
struct SV {  // device views of the Stokes field set
    DF<T> V[3], rV[3], P, divV, tau[6], tau_old[6], eta, ieta, rho[3], Tt, To, qT[3];
    // continuity forcing of the defect-correction solve: the pressure update and the divV
    // output use (divV + fP); the deviatoric strain rate uses divV alone
    DF<T> fP;
    // precomputed viscosity terms of the variable-viscosity form (bit-identical to computing
    // them in the kernel; saves the FP64 divisions): eta_ve at cells, and per shear component
    // the interpolated 1/eta and its eta_ve (2D: [0] = xy; 3D: [0..2] = xy, xz, yz)
    DF<T> eveC, ievE[3], eveE[3];
    int has_rV, has_divV, has_eta, has_ieta, has_rho[3], has_fP, has_pre;
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

// Body force per velocity component as a device FunctionField, and the grid's coordinates. A
// separate kernel argument of the two kernels that evaluate it (the velocity update and the
// FP64 defect): the march kernels keep the small SP as their scalar argument.
template <class T>
struct BodyFn {
    FnDev<T> fn[3];
    T org[3], dx[3];
};

// Body-force function of velocity component `comp` at its point (i, j, k): Vertex along comp,
// Center along the other dimensions.
template <class T>
__device__ __forceinline__ T body_fn(const BodyFn<T>& s, int comp, int nd, int i, int j, int k) {
    const int I[3] = {i, j, k};
    T x[3] = {T(0), T(0), T(0)};
    for (int e = 0; e < nd; ++e) x[e] = grid_coord(s.org[e], s.dx[e], I[e], e == comp);
    return fn_eval(s.fn[comp], nd, x);
}

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
BodyFn<T> body_fns(const cg_grid* g, const cg_stokes_params* p) {
    BodyFn<T> b;
    for (int d = 0; d < 3; ++d) {
        b.org[d] = (T)g->origin[d];
        b.dx[d] = (T)g->spacing[d];
        b.fn[d].kind = p->rho_g_fn[d].kind;
        for (int q = 0; q < 8; ++q) b.fn[d].p[q] = (T)p->rho_g_fn[d].p[q];
    }
    return b;
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

// 1/eta on the (a, b) shear edge of point I: the Linear rule over the 4 cells around it, dim a
// innermost (interpolation.jl:217-221), i.e. the harmonic average of eta.
template <class T>
__device__ __forceinline__ T shear_inv_eta(const SV<T>& v, int i, int j, int k, int a, int b) {
    const int ai = a == 0, aj = a == 1, ak = a == 2;
    const int bi = b == 0, bj = b == 1, bk = b == 2;
    const T e00 = v.inv_eta(i - ai - bi, j - aj - bj, k - ak - bk);
    const T e10 = v.inv_eta(i - bi, j - bj, k - bk);
    const T e01 = v.inv_eta(i - ai, j - aj, k - ak);
    const T e11 = v.inv_eta(i, j, k);
    const T lo = fma(T(0.5), e10 - e00, e00);
    const T hi = fma(T(0.5), e11 - e01, e01);
    return fma(T(0.5), hi - lo, lo);
}

// Operand readers of the stress and velocity kernels. NoMask reads a value; FieldMaskW is
// Chmy's FieldMask (src/GridOperators/field_mask.jl:1-117) seen by the masked operators
// (src/GridOperators/masked_operators.jl:11-39): every operand of a derivative is multiplied by
// the mask at its own location and index. `loc` is the operand's location bits (bit d set for
// Vertex along d), the index into the mask's weight fields. With unit weights both readers give
// the same bits (x * 1 == x, also under contraction into a fused multiply-add).
template <class T>
struct NoMask {
    __device__ __forceinline__ T operator()(int, const DF<T>& f, int i, int j, int k) const { return f(i, j, k); }
};
template <class T>
struct FieldMaskW {
    DF<T> w[8];
    __device__ __forceinline__ T operator()(int loc, const DF<T>& f, int i, int j, int k) const {
        return f(i, j, k) * w[loc](i, j, k);
    }
};

// Viscosity terms used by every PT iteration, computed once per solve over [0, n+1]^N with the
// stress kernel's own expressions (so the values are bit-identical).
template <class T, int ND>
__global__ void precompute_kernel(const SV<T> v, const SP<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    v.eveC(i, j, k) = T(1) / (v.inv_eta(i, j, k) + s.inv_Gdt);
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int e = 0; e < (ND == 2 ? 1 : 3); ++e) {
        const T iev = shear_inv_eta(v, i, j, k, pairs[e][0], pairs[e][1]);
        v.ievE[e](i, j, k) = iev;
        v.eveE[e](i, j, k) = T(1) / (iev + s.inv_Gdt);
    }
}

// update_stress! at one point. Tensor order 2D (xx, yy, xy), 3D (xx, yy, zz, xy, xz, yz).
// M reads the operands of the strain-rate derivatives (NoMask, or FieldMaskW for the masked
// operators ∂(V.d, ω, g, I) and divg(V, ω, g, I)); V.d sits at location bits 1 << d.
template <class T, int ND, bool WRITE_RES, class M>
__global__ void stress_kernel(const SV<T> v, const SP<T> s, int e0, int e1, const M m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const DF<T>& Vx = v.V[0];
    const DF<T>& Vy = v.V[1];
    // ∂x(V.x) at Center: V.x is Vertex in x -> V.x[i+1] - V.x[i]
    const T exx = (m(1, Vx, i + 1, j, k) - m(1, Vx, i, j, k)) * s.idx[0];
    const T eyy = (m(2, Vy, i, j + 1, k) - m(2, Vy, i, j, k)) * s.idx[1];
    T dv = exx + eyy;
    T ezz = T(0);
    if (ND > 2) {
        const DF<T>& Vz = v.V[2];
        ezz = (m(4, Vz, i, j, k + 1) - m(4, Vz, i, j, k)) * s.idx[2];
        dv = dv + ezz;
    }
    const T dvP = v.has_fP ? dv + v.fP(i, j, k) : dv;
    if (WRITE_RES && v.has_divV) v.divV(i, j, k) = dvP;
    T ieta_c = T(0), eve_c = s.eta_ve;
    if (v.has_eta) {
        ieta_c = v.inv_eta(i, j, k);
        eve_c = v.has_pre ? v.eveC(i, j, k) : T(1) / (ieta_c + s.inv_Gdt);
    }
    v.P(i, j, k) = v.P(i, j, k) - dvP * eve_c * s.dtau_Pr;
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
            T iev, eve;
            if (v.has_pre) {
                const int e = ND == 2 ? 0 : c - 3;
                iev = v.ievE[e](i, j, k);
                eve = v.eveE[e](i, j, k);
            } else {
                iev = shear_inv_eta(v, i, j, k, a, b);
                eve = T(1) / (iev + s.inv_Gdt);
            }
            const T r = -(t - to) * s.inv_Gdt - t * iev + T(2.0) * eod;
            v.tau[c](i, j, k) = t + r * eve * s.dtau_r;
        } else {  // examples/stokes_2d_inc_ve_T.jl:30
            const T r = -(t - to) / (s.G * s.dt) - t / s.eta + T(2.0) * eod;
            v.tau[c](i, j, k) = t + r * s.eta_ve * s.dtau_r;
        }
    };
    // ∂y(V.x) at the xy vertex: V.x is Center in y -> V.x[j] - V.x[j-1]
    const T exy = T(0.5) * ((m(1, Vx, i, j, k) - m(1, Vx, i, j - 1, k)) * s.idx[1] +
                            (m(2, Vy, i, j, k) - m(2, Vy, i - 1, j, k)) * s.idx[0]);
    if (ND == 2) {
        diag(0, exx);
        diag(1, eyy);
        shear(2, exy, 0, 1);
    } else {
        const DF<T>& Vz = v.V[2];
        const T exz = T(0.5) * ((m(1, Vx, i, j, k) - m(1, Vx, i, j, k - 1)) * s.idx[2] +
                                (m(4, Vz, i, j, k) - m(4, Vz, i - 1, j, k)) * s.idx[0]);
        const T eyz = T(0.5) * ((m(2, Vy, i, j, k) - m(2, Vy, i, j, k - 1)) * s.idx[2] +
                                (m(4, Vz, i, j, k) - m(4, Vz, i, j - 1, k)) * s.idx[1]);
        diag(0, exx);
        diag(1, eyy);
        diag(2, ezz);
        shear(3, exy, 0, 1);
        shear(4, exz, 0, 2);
        shear(5, eyz, 1, 2);
    }
}

// update_velocity! at one point. M reads the operands of the pressure and stress derivatives
// (P and τ_dd at location bits 0, τ_xy 3, τ_xz 5, τ_yz 6).
template <class T, int ND, bool WRITE_RES, class M>
__global__ void velocity_kernel(const SV<T> v, const SP<T> s, const BodyFn<T> bf, int e0, int e1, const M m) {
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
    const int LXY = 3, LXZ = 5, LYZ = 6;  // location bits of the shear components
    T rx = -((m(0, P, i, j, k) - m(0, P, i - 1, j, k)) * s.idx[0]) + (m(0, txx, i, j, k) - m(0, txx, i - 1, j, k)) * s.idx[0];
    rx = rx + (m(LXY, txy, i, j + 1, k) - m(LXY, txy, i, j, k)) * s.idx[1];
    T ry = -((m(0, P, i, j, k) - m(0, P, i, j - 1, k)) * s.idx[1]) + (m(0, tyy, i, j, k) - m(0, tyy, i, j - 1, k)) * s.idx[1];
    ry = ry + (m(LXY, txy, i + 1, j, k) - m(LXY, txy, i, j, k)) * s.idx[0];
    T rz = T(0);
    if (ND > 2) {
        const DF<T>& tzz = v.tau[2];
        const DF<T>& txz = v.tau[4];
        const DF<T>& tyz = v.tau[5];
        rx = rx + (m(LXZ, txz, i, j, k + 1) - m(LXZ, txz, i, j, k)) * s.idx[2];
        ry = ry + (m(LYZ, tyz, i, j, k + 1) - m(LYZ, tyz, i, j, k)) * s.idx[2];
        rz = -((m(0, P, i, j, k) - m(0, P, i, j, k - 1)) * s.idx[2]) + (m(0, tzz, i, j, k) - m(0, tzz, i, j, k - 1)) * s.idx[2];
        rz = rz + (m(LXZ, txz, i + 1, j, k) - m(LXZ, txz, i, j, k)) * s.idx[0];
        rz = rz + (m(LYZ, tyz, i, j + 1, k) - m(LYZ, tyz, i, j, k)) * s.idx[1];
    }
    if (v.has_rho[0]) rx = rx - v.rho[0](i, j, k);
    else if (bf.fn[0].kind) rx = rx - body_fn(bf, 0, ND, i, j, k);
    if (v.has_rho[1]) ry = ry - v.rho[1](i, j, k);
    else if (bf.fn[1].kind) ry = ry - body_fn(bf, 1, ND, i, j, k);
    if (ND > 2 && v.has_rho[2]) rz = rz - v.rho[2](i, j, k);
    else if (ND > 2 && bf.fn[2].kind) rz = rz - body_fn(bf, 2, ND, i, j, k);
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

// ---- fused thermal step: update_thermal_flux! + update_thermal! ------------------------------
//
// T_out = T_old - dt * divg(qT) with qT_d = -lambda * d_d(T) + max(V_d, 0) * T_left +
// min(V_d, 0) * T_right (examples/stokes_2d_inc_ve_T.jl:35-50, 3D :59-77) computed on the fly
// at the two faces of each cell, over Chmy's launch range. A face flux at index n+2 lies beyond
// the flux kernel's launch range, so in the two-kernel form it reads the untouched allocation:
// zero here. Every operation is rounded once in the oracle's order (max/min as std::max/min).
template <class T>
__device__ __forceinline__ T heat_flux(T mlam, T tl, T tr, T v, T idx) {
    const T vp = v < T(0) ? T(0) : v;  // std::max(v, 0)
    const T vm = T(0) < v ? T(0) : v;  // std::min(v, 0)
    return radd(radd(rmul(mlam, rmul(rsub(tr, tl), idx)), rmul(vp, tl)), rmul(vm, tr));
}

template <class T>
struct ThermalStep {
    DF<T> Tin, Told, Tout, V[3];
    T mlam, dt, idx[3];
};

template <class T, int ND>
__global__ void thermal_step_kernel(const ThermalStep<T> a, int e0, int e1, int e2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const T c = a.Tin(i, j, k);
    const T qx0 = heat_flux(a.mlam, a.Tin(i - 1, j, k), c, a.V[0](i, j, k), a.idx[0]);
    const T qx1 = i + 1 <= e0 ? heat_flux(a.mlam, c, a.Tin(i + 1, j, k), a.V[0](i + 1, j, k), a.idx[0]) : T(0);
    T dq = rmul(rsub(qx1, qx0), a.idx[0]);
    const T qy0 = heat_flux(a.mlam, a.Tin(i, j - 1, k), c, a.V[1](i, j, k), a.idx[1]);
    const T qy1 = j + 1 <= e1 ? heat_flux(a.mlam, c, a.Tin(i, j + 1, k), a.V[1](i, j + 1, k), a.idx[1]) : T(0);
    dq = radd(dq, rmul(rsub(qy1, qy0), a.idx[1]));
    if (ND > 2) {
        const T qz0 = heat_flux(a.mlam, a.Tin(i, j, k - 1), c, a.V[2](i, j, k), a.idx[2]);
        const T qz1 = k + 1 <= e2 ? heat_flux(a.mlam, c, a.Tin(i, j, k + 1), a.V[2](i, j, k + 1), a.idx[2]) : T(0);
        dq = radd(dq, rmul(rsub(qz1, qz0), a.idx[2]));
    }
    a.Tout(i, j, k) = rsub(a.Told(i, j, k), rmul(a.dt, dq));
}

// ---- bc!(V) folded into the velocity reads of the marching kernels -------------------------
//
// A PT iteration ends with bc!(V) (examples/stokes_2d_inc_ve_T.jl:81-89): its boundary planes
// are functions of the interior the iteration just wrote. The marching kernel can instead read
// the unpatched velocity of the previous iteration and apply the same rules to each value it
// uses, which leaves one boundary-condition launch at the end of a run of iterations instead
// of one per iteration. The rules are those of cg_bc_apply for Dirichlet and Neumann kinds
// (Chmy's FirstOrderBC): per velocity component a, dimension d and side s, the planes g (an
// index along d) become a constant (Dirichlet on a Vertex dimension), 2 v - F[src]
// (Dirichlet on a Center dimension) or F[src] -/+ h v (Neumann), applied over the tangential
// range 0..n+2, dimension y (then z in 3D) before x, side 0 before side 1, with the same
// fused multiply-adds, so the folded value equals the patched one bit for bit. Periodic
// kinds are not folded. A value the later phase reads (a corner) is the earlier phase's
// result, exactly as in the chain the boundary-condition kernel walks.
enum { FOLD_NONE = 0, FOLD_CONST = 1, FOLD_DIRC = 2, FOLD_NEU = 3 };

template <class T>
struct VFold {
    int on;
    signed char rule[3][3][2];  // [component][dimension][side]
    int g[3][3][2], src[3][3][2];
    T val[3][3][2];             // Dirichlet value; Neumann: -v on side 0, +v on side 1
    T h[3];
    int lim[3];                 // tangential range 0..n+2 of each dimension
};

template <class T>
__device__ __forceinline__ T fold_rule(int r, T base, T v, T h) {
    return r == FOLD_DIRC ? rfma(T(2), rsub(v, base), base) : rfma(h, v, base);
}

// The rules of cg_bc_apply for velocity component a (Vertex along a, Center along the others)
// of a grid with n[d] cells. Returns false when a kind cannot be folded (periodic).
template <class T>
inline bool make_vfold(const cg_grid* g, const cg_bc* bc_V, VFold<T>* out) {
    std::memset(out, 0, sizeof(*out));
    if (!bc_V) return false;
    const int nd = g->ndim;
    for (int d = 0; d < nd; ++d) {
        out->h[d] = (T)g->spacing[d];
        out->lim[d] = g->n[d] + 2;
    }
    for (int a = 0; a < nd; ++a)
        for (int d = 0; d < nd; ++d) {
            const bool vtx = d == a;
            const int ext = vtx ? g->n[d] + 1 : g->n[d];
            for (int s = 0; s < 2; ++s) {
                if (bc_V[a].values[d][s]) return false;  // per-point values: not folded
                const T v = (T)bc_V[a].value[d][s];
                signed char& r = out->rule[a][d][s];
                switch (bc_V[a].kind[d][s]) {
                    case CG_BC_NONE: r = FOLD_NONE; break;
                    case CG_BC_DIRICHLET:
                        if (vtx) {
                            r = FOLD_CONST;
                            out->g[a][d][s] = s ? ext : 1;
                        } else {
                            r = FOLD_DIRC;
                            out->g[a][d][s] = s ? ext + 1 : 0;
                            out->src[a][d][s] = s ? ext : 1;
                        }
                        out->val[a][d][s] = v;
                        break;
                    case CG_BC_NEUMANN:
                        r = FOLD_NEU;
                        out->g[a][d][s] = s ? ext + 1 : 0;
                        out->src[a][d][s] = s ? ext : 1;
                        out->val[a][d][s] = s ? v : -v;
                        break;
                    default: return false;
                }
            }
        }
    out->on = 1;
    return true;
}

// ---- fused 2D PT iteration (variable viscosity): update_stress! + update_velocity! -----------
//
// One launch per PT iteration, reading the `in` buffers and writing the `out` buffers
// (ping-pong). Points outside Chmy's launch range [0, n+1] keep their old values, exactly as in
// the two-kernel form.
template <class T>
struct Fused2D {
    DF<T> Vx_in, Vy_in, Vx_out, Vy_out;
    DF<T> txx_in, tyy_in, txy_in, txx_out, tyy_out, txy_out, P_in, P_out;
    DF<T> txx_o, tyy_o, txy_o, ieta, fP, rhox, rhoy, divV, rVx, rVy;
    int has_fP, has_rho;
    VFold<T> bc;  // bc.on: the V_in values are read through bc!(V)
};

// ---- warp-marching fused 2D PT iteration --------------------------------------------------
//
// update_stress! followed by update_velocity! in one launch, without shared memory. It writes
// the new P, tau_xx, tau_yy, tau_xy and V on [0, n+1]^2 (and divV, r_V when asked); points
// outside that range keep the values the out buffers hold. A warp owns 30
// launch columns i = c0 .. c0+29 and a segment of rows js .. je. Lane l holds column
// c0 - 1 + l, so lanes 0 and 31 are one-column halos. Each lane reads every input of its
// column once per row; x-neighbours come from shuffles. The warp then marches up the rows,
// keeping in registers the previous row's velocity, 1/eta and the new P, tau_yy and tau_xy.
// Iteration j computes the new cell row j and vertex row j+1, then the velocity of row j.
// The segment's prologue computes cell row js-1 and vertex row js.
//
// Shuffle validity: a cell at lane l needs Vx of lane l+1, so lane 31's cell is invalid; a
// vertex at lane l needs Vy and 1/eta of lane l-1, so lane 0's vertex is invalid. The owned
// lanes 1..30 read cells of lanes l-1, l and vertices of lanes l, l+1, all valid.
// Ix is the element-offset type: int where every offset fits in 32 bits, else long.
template <class T, class Ix, bool UNI>
struct MAt {  // column i of a lane; UNI: every array has the row stride s1u
    int i;
    Ix s1u;
    __device__ __forceinline__ Ix off(const DF<T>& f, int j) const { return (Ix)i + (Ix)j * (UNI ? s1u : (Ix)f.s1); }
    __device__ __forceinline__ T ld(const DF<T>& f, int j, bool ok) const { return ok ? __ldg(f.p + off(f, j)) : T(0); }
    __device__ __forceinline__ void st(const DF<T>& f, int j, T v) const { f.p[off(f, j)] = v; }
};

// Inputs of one marching step at column i: row j+1 of the vertex-row inputs, row j of the
// cell-row inputs.
template <class T>
struct MarchRow {
    T Vx, Vy, ie, txy, txyo;                   // row j+1
    T P, txx, tyy, txo, tyo, fp, rhox, rhoy;  // row j
};

template <class T, class Ix, bool UNI>
__device__ __forceinline__ MarchRow<T> march_load(const Fused2D<T>& f, const MAt<T, Ix, UNI>& at, int j, int e1,
                                                  bool inV, bool inC) {
    MarchRow<T> r;
    const int jn = j + 1;
    const bool vn = inV && jn <= e1 + 1;
    r.Vx = at.ld(f.Vx_in, jn, vn);
    r.Vy = at.ld(f.Vy_in, jn, vn);
    r.ie = at.ld(f.ieta, jn, vn);
    r.txy = at.ld(f.txy_in, jn, vn);
    r.txyo = at.ld(f.txy_o, jn, inC && jn <= e1);
    const bool c = inC && j <= e1;
    r.P = at.ld(f.P_in, j, c);
    r.txx = at.ld(f.txx_in, j, c);
    r.tyy = at.ld(f.tyy_in, j, c);
    r.txo = at.ld(f.txx_o, j, c);
    r.tyo = at.ld(f.tyy_o, j, c);
    r.fp = f.has_fP ? at.ld(f.fP, j, c) : T(0);
    r.rhox = f.has_rho ? at.ld(f.rhox, j, c) : T(0);
    r.rhoy = f.has_rho ? at.ld(f.rhoy, j, c) : T(0);
    return r;
}

// Velocity component a at column i, row j of a marching warp, read through bc!(V), in two
// steps. fold_y (rows; the caller tests that row j can hold a y-plane, uniformly in the warp):
// v is the stored value, vprev the folded value of row j-1 and vnext the stored value of row
// j+1. A y-plane's source row is always the adjacent one (row 0 from row 1, row n+1 from n,
// row n+2 from n+1; rows 1 and n+1 of a Vertex dimension are constants) and never a y-plane
// itself. The previous row's folded value equals its stored one except in an x-plane column,
// where fold_x overrides the y result anyway.
template <class T>
__device__ __forceinline__ T fold_y(const VFold<T>& b, int a, int i, int j, T v, T vprev, T vnext) {
    if (i >= 0 && i <= b.lim[0]) {
        const int r0 = b.rule[a][1][0], r1 = b.rule[a][1][1];
        if (r0 != FOLD_NONE && j == b.g[a][1][0])
            v = r0 == FOLD_CONST ? b.val[a][1][0] : fold_rule(r0, vnext, b.val[a][1][0], b.h[1]);
        if (r1 != FOLD_NONE && j == b.g[a][1][1])
            v = r1 == FOLD_CONST ? b.val[a][1][1] : fold_rule(r1, vprev, b.val[a][1][1], b.h[1]);
    }
    return v;
}

// fold_x (columns; called by the whole warp when its strip holds an x-plane, for a row in the
// tangential range 0..n+2): an x-plane takes its neighbour lane's y-folded value. Lanes 0 and
// 31 are halos: a left plane (column 0 or 1) sits at lane >= 1 with its source one lane up, a
// right plane (column n+1 or n+2) at lane >= 1 of any strip that owns a column, its source one
// lane down.
template <class T>
__device__ __forceinline__ T fold_x(const VFold<T>& b, int a, int i, T v) {
    constexpr unsigned FULL = 0xffffffffu;
    const int r0 = b.rule[a][0][0], r1 = b.rule[a][0][1];
    T vr = v, vl = v;
    if (r0 > FOLD_CONST || r1 > FOLD_CONST) {  // a rule with a source: the neighbours' values
        vr = __shfl_down_sync(FULL, v, 1);
        vl = __shfl_up_sync(FULL, v, 1);
    }
    if (r0 != FOLD_NONE && i == b.g[a][0][0])
        v = r0 == FOLD_CONST ? b.val[a][0][0] : fold_rule(r0, vr, b.val[a][0][0], b.h[0]);
    if (r1 != FOLD_NONE && i == b.g[a][0][1])
        v = r1 == FOLD_CONST ? b.val[a][0][1] : fold_rule(r1, vl, b.val[a][0][1], b.h[0]);
    return v;
}

// -(t - t_old) * inv_Gdt - t * ieta + 2 * e: the VE stress residual, left to right.
template <class T>
__device__ __forceinline__ T stress_res(const SP<T>& s, T t, T to, T ie, T e) {
    return radd(rsub(rmul(-rsub(t, to), s.inv_Gdt), rmul(t, ie)), rmul(T(2.0), e));
}

template <class T>
struct CellNew {
    T P, txx, tyy, dvP;
};

// New P, tau_xx, tau_yy at cell (i, j) from Vx(i, j), Vx(i+1, j), Vy(i, j), Vy(i, j+1) and the
// cell's inputs (update_stress!, variable-viscosity form).
template <class T>
__device__ __forceinline__ CellNew<T> march_cell(const SP<T>& s, bool has_fP, T vx, T vxR, T vy, T vyU, T ie, T P,
                                                 T txx, T txo, T tyy, T tyo, T fp) {
    const T exx = rmul(rsub(vxR, vx), s.idx[0]);
    const T eyy = rmul(rsub(vyU, vy), s.idx[1]);
    const T dv = radd(exx, eyy);
    const T dvt = rmul(dv, s.third);
    const T eve = rrcp(radd(ie, s.inv_Gdt));
    CellNew<T> c;
    c.dvP = has_fP ? radd(dv, fp) : dv;
    c.P = rsub(P, rmul(rmul(c.dvP, eve), s.dtau_Pr));
    c.txx = radd(txx, rmul(rmul(stress_res(s, txx, txo, ie, rsub(exx, dvt)), eve), s.dtau_r));
    c.tyy = radd(tyy, rmul(rmul(stress_res(s, tyy, tyo, ie, rsub(eyy, dvt)), eve), s.dtau_r));
    return c;
}

// New tau_xy at vertex (i, jv) from Vx(i, jv-1), Vx(i, jv), Vy(i-1, jv), Vy(i, jv) and the four
// cells' 1/eta around it (e00 = (i-1, jv-1), e10 = (i, jv-1), e01 = (i-1, jv), e11 = (i, jv)),
// interpolated with the Linear rule, x innermost.
template <class T>
__device__ __forceinline__ T march_vertex(const SP<T>& s, T vx0, T vx1, T vyl, T vy, T e00, T e10, T e01, T e11,
                                          T t2, T o2) {
    const T half = T(0.5);
    const T exy = rmul(half, radd(rmul(rsub(vx1, vx0), s.idx[1]), rmul(rsub(vy, vyl), s.idx[0])));
    const T lo = rfma(half, rsub(e10, e00), e00);
    const T hi = rfma(half, rsub(e11, e01), e01);
    const T iev = rfma(half, rsub(hi, lo), lo);
    const T eve = rrcp(radd(iev, s.inv_Gdt));
    return radd(t2, rmul(rmul(stress_res(s, t2, o2, iev, exy), eve), s.dtau_r));
}

template <class T, class Ix, bool UNI, bool WRITE_RES, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) march2d_kernel(const Fused2D<T> f, const SP<T> s, int e0, int e1,
                                                            int nstrip, int nwarps, int seg_rows, long s1u) {
    constexpr unsigned FULL = 0xffffffffu;
    cg_dep_wait();
    cg_dep_release();
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (gw >= nwarps) return;  // whole warp
    const int strip = gw % nstrip;
    const int js = (gw / nstrip) * seg_rows;
    if (js > e1) return;  // whole warp
    const int je = min(js + seg_rows - 1, e1);
    const int i = strip * 30 - 1 + lane;
    const MAt<T, Ix, UNI> at{i, (Ix)s1u};
    const bool own = lane >= 1 && lane <= 30 && i <= e0;
    const bool inV = i <= e0 + 1;  // V, 1/eta, tau_xy readable
    const bool inC = i <= e0;      // cell inputs, tau_xy_old readable
    const bool oldcell = i < 0;    // column -1 keeps its old cell values
    // bc!(V) folded into the reads: the strip holds an x-plane (columns 0, 1, n+1, n+2) / the
    // rows js-1 .. je+1 hold a y-plane (rows 0, 1, n+1, n+2)
    const bool xb = f.bc.on && (strip == 0 || strip * 30 + 30 >= e0);
    const bool ylow = js <= 2, yhigh = je + 2 >= e1;
    const bool yb = f.bc.on && (ylow || yhigh);
    // rows ylo..yhi of the marching steps can hold a y-plane (0..1, n+1..n+2, or all)
    const int ylo = ylow ? 0 : e1, yhi = yhigh ? e1 + 1 : 1;

    // ---- prologue: new cell row js-1 (P and tau_yy only) and new vertex row js ----
    T Vx_c, Vy_c, ie_c, ieL_c, ie_p, Pn_p, Tyyn_p, txy_c;
    MarchRow<T> cur;
    {
        const int jp = js - 1;  // >= -1
        T vxp = at.ld(f.Vx_in, jp, inV);
        T vyp = at.ld(f.Vy_in, jp, inV);
        const T iep = at.ld(f.ieta, jp, inV);
        const T pp = at.ld(f.P_in, jp, inC);
        const T typ = at.ld(f.tyy_in, jp, inC);
        const T tyop = at.ld(f.tyy_o, jp, inC);
        const T fpp = f.has_fP ? at.ld(f.fP, jp, inC) : T(0);
        Vx_c = at.ld(f.Vx_in, js, inV);
        Vy_c = at.ld(f.Vy_in, js, inV);
        ie_c = at.ld(f.ieta, js, inV);
        const T t2 = at.ld(f.txy_in, js, inV);
        const T o2 = at.ld(f.txy_o, js, inC);
        // the first marching step's loads (row js+1) are issued before the prologue computes
        cur = march_load(f, at, js, e1, inV, inC);
        if (yb) {
            // row js+1 is the source of a plane at row js = 0; row js-1 can be no side-1 plane
            vxp = fold_y(f.bc, 0, i, jp, vxp, T(0), Vx_c);
            vyp = fold_y(f.bc, 1, i, jp, vyp, T(0), Vy_c);
        }
        if (xb && jp >= 0) {
            vxp = fold_x(f.bc, 0, i, vxp);
            vyp = fold_x(f.bc, 1, i, vyp);
        }
        if (yb) {
            Vx_c = fold_y(f.bc, 0, i, js, Vx_c, vxp, cur.Vx);
            Vy_c = fold_y(f.bc, 1, i, js, Vy_c, vyp, cur.Vy);
        }
        if (xb) {
            Vx_c = fold_x(f.bc, 0, i, Vx_c);
            Vy_c = fold_x(f.bc, 1, i, Vy_c);
        }
        // cell (i, js-1); row -1 and column -1 keep their old values
        const T vxpR = __shfl_down_sync(FULL, vxp, 1);
        const CellNew<T> cp = march_cell(s, f.has_fP != 0, vxp, vxpR, vyp, Vy_c, iep, pp, T(0), T(0), typ, tyop, fpp);
        const bool keep = jp < 0 || oldcell;
        Pn_p = keep ? pp : cp.P;
        Tyyn_p = keep ? typ : cp.tyy;
        // vertex (i, js)
        const T vyL = __shfl_up_sync(FULL, Vy_c, 1);
        const T iepL = __shfl_up_sync(FULL, iep, 1);
        ieL_c = __shfl_up_sync(FULL, ie_c, 1);
        txy_c = (i > e0) ? t2 : march_vertex(s, vxp, Vx_c, vyL, Vy_c, iepL, iep, ieL_c, ie_c, t2, o2);
        if (own) at.st(f.txy_out, js, txy_c);
        ie_p = iep;
    }

    // the next row's loads are issued before the current row is computed
    for (int j = js; j <= je; ++j) {
        MarchRow<T> nxt;
        if (j < je) nxt = march_load(f, at, j + 1, e1, inV, inC);
        // row j+1 in 1..n+2: a side-0 y-plane there is a constant (row 1 of a Vertex dimension)
        if (yb && j + 1 >= ylo && j + 1 <= yhi) {
            cur.Vx = fold_y(f.bc, 0, i, j + 1, cur.Vx, Vx_c, T(0));
            cur.Vy = fold_y(f.bc, 1, i, j + 1, cur.Vy, Vy_c, T(0));
        }
        if (xb) {
            cur.Vx = fold_x(f.bc, 0, i, cur.Vx);
            cur.Vy = fold_x(f.bc, 1, i, cur.Vy);
        }
        // new cell (i, j)
        const T vxR = __shfl_down_sync(FULL, Vx_c, 1);
        CellNew<T> c = march_cell(s, f.has_fP != 0, Vx_c, vxR, Vy_c, cur.Vy, ie_c, cur.P, cur.txx, cur.txo, cur.tyy,
                                  cur.tyo, cur.fp);
        if (oldcell) {
            c.P = cur.P;
            c.txx = cur.txx;
            c.tyy = cur.tyy;
        }
        // new vertex (i, j+1)
        const T vyL = __shfl_up_sync(FULL, cur.Vy, 1);
        const T ieL_n = __shfl_up_sync(FULL, cur.ie, 1);
        const T tn = (i > e0 || j + 1 > e1)
                         ? cur.txy
                         : march_vertex(s, Vx_c, cur.Vx, vyL, cur.Vy, ieL_c, ie_c, ieL_n, cur.ie, cur.txy, cur.txyo);
        // velocity (i, j): r_V = -d(P) + d(tau_dd) + d(tau_xy) - rho g, left to right
        const T PL = __shfl_up_sync(FULL, c.P, 1);
        const T TxxL = __shfl_up_sync(FULL, c.txx, 1);
        const T txyR = __shfl_down_sync(FULL, txy_c, 1);
        if (own) {
            T rx = radd(-rmul(rsub(c.P, PL), s.idx[0]), rmul(rsub(c.txx, TxxL), s.idx[0]));
            rx = radd(rx, rmul(rsub(tn, txy_c), s.idx[1]));
            T ry = radd(-rmul(rsub(c.P, Pn_p), s.idx[1]), rmul(rsub(c.tyy, Tyyn_p), s.idx[1]));
            ry = radd(ry, rmul(rsub(txyR, txy_c), s.idx[0]));
            if (f.has_rho) {
                rx = rsub(rx, cur.rhox);
                ry = rsub(ry, cur.rhoy);
            }
            at.st(f.P_out, j, c.P);
            at.st(f.txx_out, j, c.txx);
            at.st(f.tyy_out, j, c.tyy);
            if (j + 1 <= je) at.st(f.txy_out, j + 1, tn);
            if (WRITE_RES) {
                at.st(f.divV, j, c.dvP);
                at.st(f.rVx, j, rx);
                at.st(f.rVy, j, ry);
            }
            at.st(f.Vx_out, j, radd(Vx_c, rmul(rx, rmul(s.nu_dtau, radd(fmin(ieL_c, ie_c), s.inv_Gdt)))));
            at.st(f.Vy_out, j, radd(Vy_c, rmul(ry, rmul(s.nu_dtau, radd(fmin(ie_p, ie_c), s.inv_Gdt)))));
        }
        // advance one row
        Vx_c = cur.Vx;
        Vy_c = cur.Vy;
        ie_p = ie_c;
        ie_c = cur.ie;
        ieL_c = ieL_n;
        Pn_p = c.P;
        Tyyn_p = c.tyy;
        txy_c = tn;
        cur = nxt;
    }
}

// ---- two PT iterations per pass (temporal blocking) -----------------------------------------
//
// march2d_x2_kernel takes two consecutive iterations of march2d_kernel in one pass over the
// rows. Stage A is the first iteration: it reads the `in` buffers (through bc!(V) when f.bc.on
// and fold_a) as march2d_kernel does and keeps its results in registers. Stage B is the second:
// it reads A's results two rows behind A (through bc!(V) when f.bc.on, since A's velocities are
// the ones bc!(V) would patch) and the constant inputs, and writes the `out` buffers. A pass
// moves the bytes of one iteration for two. A warp owns 28 columns: lane l holds column
// c0 - 2 + l. A's results are valid on lanes 1..30, B's on the owned lanes 2..29. A marches rows
// js-2 .. je+1 and B rows js-1 .. je; each stage's first row only starts its state.
// Points outside the launch range [0, n+1] keep their values: A passes its inputs on there (the
// two-launch sequence passes on the intermediate buffer's values, which are the input buffer's
// wherever the two buffers agree outside the launch range, as the callers' pairs do), and B
// leaves the out buffers untouched there. Every operation is march2d_kernel's, in its order,
// so a pass equals two launches of it bit for bit.

// Marching state of one iteration at the current row j: V of row j (through bc!(V)), 1/eta of
// row j (own lane and left lane) and of row j-1, the new P and tau_yy of cell row j-1 and the
// new tau_xy of vertex row j.
template <class T>
struct MState {
    T Vx, Vy, ie, ieL, ie_p, Pn_p, Tyyn_p, txy;
};

// Results of one step at row j: new cell row j, new vertex row j+1, new velocity of row j (its
// input outside the launch range) and the momentum residuals of row j.
template <class T>
struct MStep {
    CellNew<T> c;
    T tn, vx, vy, rx, ry;
};

// One step of one iteration at row j: the body of march2d_kernel's loop. cur holds row j+1's
// vertex inputs (Vx, Vy as stored) and row j's cell inputs; vnx, vny are row j+2's stored
// velocities (the source of a plane at row j+1 = 0). st advances to row j+1.
template <class T>
__device__ __forceinline__ MStep<T> x2_step(const Fused2D<T>& f, const SP<T>& s, MState<T>& st, MarchRow<T>& cur,
                                           T vnx, T vny, int i, int j, int e0, int e1, bool xfold, bool yfold, int ylo,
                                           int yhi) {
    constexpr unsigned FULL = 0xffffffffu;
    if (yfold && j + 1 >= ylo && j + 1 <= yhi) {
        cur.Vx = fold_y(f.bc, 0, i, j + 1, cur.Vx, st.Vx, vnx);
        cur.Vy = fold_y(f.bc, 1, i, j + 1, cur.Vy, st.Vy, vny);
    }
    if (xfold && j + 1 >= 0 && j + 1 <= e1 + 1) {  // x-planes over the tangential rows 0..n+2
        cur.Vx = fold_x(f.bc, 0, i, cur.Vx);
        cur.Vy = fold_x(f.bc, 1, i, cur.Vy);
    }
    MStep<T> o;
    // new cell (i, j)
    const T vxR = __shfl_down_sync(FULL, st.Vx, 1);
    o.c = march_cell(s, f.has_fP != 0, st.Vx, vxR, st.Vy, cur.Vy, st.ie, cur.P, cur.txx, cur.txo, cur.tyy, cur.tyo,
                     cur.fp);
    const bool in_range = i >= 0 && i <= e0 && j >= 0 && j <= e1;
    if (!in_range) {
        o.c.P = cur.P;
        o.c.txx = cur.txx;
        o.c.tyy = cur.tyy;
    }
    // new vertex (i, j+1)
    const T vyL = __shfl_up_sync(FULL, cur.Vy, 1);
    const T ieL_n = __shfl_up_sync(FULL, cur.ie, 1);
    o.tn = (i < 0 || i > e0 || j + 1 < 0 || j + 1 > e1)
               ? cur.txy
               : march_vertex(s, st.Vx, cur.Vx, vyL, cur.Vy, st.ieL, st.ie, ieL_n, cur.ie, cur.txy, cur.txyo);
    // velocity (i, j): r_V = -d(P) + d(tau_dd) + d(tau_xy) - rho g, left to right
    const T PL = __shfl_up_sync(FULL, o.c.P, 1);
    const T TxxL = __shfl_up_sync(FULL, o.c.txx, 1);
    const T txyR = __shfl_down_sync(FULL, st.txy, 1);
    T rx = radd(-rmul(rsub(o.c.P, PL), s.idx[0]), rmul(rsub(o.c.txx, TxxL), s.idx[0]));
    rx = radd(rx, rmul(rsub(o.tn, st.txy), s.idx[1]));
    T ry = radd(-rmul(rsub(o.c.P, st.Pn_p), s.idx[1]), rmul(rsub(o.c.tyy, st.Tyyn_p), s.idx[1]));
    ry = radd(ry, rmul(rsub(txyR, st.txy), s.idx[0]));
    if (f.has_rho) {
        rx = rsub(rx, cur.rhox);
        ry = rsub(ry, cur.rhoy);
    }
    o.rx = rx;
    o.ry = ry;
    o.vx = in_range ? radd(st.Vx, rmul(rx, rmul(s.nu_dtau, radd(fmin(st.ieL, st.ie), s.inv_Gdt)))) : st.Vx;
    o.vy = in_range ? radd(st.Vy, rmul(ry, rmul(s.nu_dtau, radd(fmin(st.ie_p, st.ie), s.inv_Gdt)))) : st.Vy;
    // advance one row
    st.Vx = cur.Vx;
    st.Vy = cur.Vy;
    st.ie_p = st.ie;
    st.ie = cur.ie;
    st.ieL = ieL_n;
    st.Pn_p = o.c.P;
    st.Tyyn_p = o.c.tyy;
    st.txy = o.tn;
    return o;
}

template <class T, class Ix, bool UNI, bool WRITE_RES, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) march2d_x2_kernel(const Fused2D<T> f, const SP<T> s, int e0, int e1,
                                                               int nstrip, int nwarps, int seg_rows, long s1u,
                                                               int fold_a) {
    constexpr unsigned FULL = 0xffffffffu;
    cg_dep_wait();
    cg_dep_release();
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (gw >= nwarps) return;  // whole warp
    const int strip = gw % nstrip;
    const int js = (gw / nstrip) * seg_rows;
    if (js > e1) return;  // whole warp
    const int je = min(js + seg_rows - 1, e1);
    const int i = strip * 28 - 2 + lane;  // >= -2: column -2 lies outside the arrays, never read
    const MAt<T, Ix, UNI> at{i, (Ix)s1u};
    const bool own = lane >= 2 && lane <= 29 && i <= e0;
    const bool inV = i >= -1 && i <= e0 + 1;  // V, 1/eta, tau_xy readable
    const bool inC = i >= -1 && i <= e0;      // cell inputs, tau_xy_old readable
    // bc!(V) folded into the reads: the strip holds an x-plane / the rows js-3 .. je+3 hold a y-plane
    const bool bcon = f.bc.on != 0;
    const bool xb = bcon && (strip == 0 || strip * 28 + 30 >= e0);
    const bool ylow = js <= 3, yhigh = je + 3 >= e1;
    const bool yb = bcon && (ylow || yhigh);
    const int ylo = ylow ? 0 : e1, yhi = yhigh ? e1 + 1 : 1;
    const bool xa = xb && fold_a, ya = yb && fold_a;
    // row j's cell inputs and row j+1's vertex inputs; rows below -1 read as zero (the first
    // segment's first row is -2)
    auto load = [&](int j) { return march_load(f, at, j, e1, inV && j >= -2, inC && j >= -1); };

    // stage A's state at row js-2. Segments start at 0 or at >= 4, so no y-plane lies on rows
    // js-2 and js-1; the velocity of the first row of each stage is discarded, so its inputs
    // from rows below are not needed.
    MState<T> a;
    {
        const int j0 = js - 2;
        const bool ok = j0 >= -1;
        a.Vx = at.ld(f.Vx_in, j0, inV && ok);
        a.Vy = at.ld(f.Vy_in, j0, inV && ok);
        a.ie = at.ld(f.ieta, j0, inV && ok);
        if (xa && j0 >= 0) {
            a.Vx = fold_x(f.bc, 0, i, a.Vx);
            a.Vy = fold_x(f.bc, 1, i, a.Vy);
        }
        a.ieL = __shfl_up_sync(FULL, a.ie, 1);
        a.ie_p = a.Pn_p = a.Tyyn_p = a.txy = T(0);
    }
    MState<T> b;
    b.Vx = b.Vy = b.ie = b.ieL = b.ie_p = b.Pn_p = b.Tyyn_p = b.txy = T(0);
    MarchRow<T> cur = load(js - 2);
    // A's results queued for B: velocity of the previous row, cells and vertices of two rows
    T qVx = T(0), qVy = T(0), qT1 = T(0), qT2 = T(0);
    CellNew<T> qC1, qC2;
    qC1.P = qC1.txx = qC1.tyy = qC1.dvP = T(0);
    qC2 = qC1;
    for (int ja = js - 2; ja <= je + 2; ++ja) {
        const bool astep = ja <= je + 1;
        const bool more = ja + 1 <= je + 1;
        MarchRow<T> nxt;
        if (more) nxt = load(ja + 1);
        const int jb = ja - 2;
        const bool bstep = jb >= js - 1;
        // B's constant inputs: row jb+1's 1/eta and tau_xy_old, row jb's cell inputs
        MarchRow<T> cb;
        if (bstep) {
            const int jn = jb + 1;
            cb.ie = at.ld(f.ieta, jn, inV && jn <= e1 + 1);
            cb.txyo = at.ld(f.txy_o, jn, inC && jn <= e1);
            const bool c = inC && jb <= e1;
            cb.txo = at.ld(f.txx_o, jb, c);
            cb.tyo = at.ld(f.tyy_o, jb, c);
            cb.fp = f.has_fP ? at.ld(f.fP, jb, c) : T(0);
            cb.rhox = f.has_rho ? at.ld(f.rhox, jb, c) : T(0);
            cb.rhoy = f.has_rho ? at.ld(f.rhoy, jb, c) : T(0);
        }
        MStep<T> oa;
        if (astep) {
            oa = x2_step(f, s, a, cur, more ? nxt.Vx : T(0), more ? nxt.Vy : T(0), i, ja, e0, e1, xa, ya, ylo, yhi);
        } else {
            oa.vx = oa.vy = oa.tn = oa.rx = oa.ry = T(0);
            oa.c = qC1;
        }
        if (ja == js - 1) {  // B's state at row js-1: A's velocity there
            b.Vx = oa.vx;
            b.Vy = oa.vy;
            if (xb && ja >= 0) {
                b.Vx = fold_x(f.bc, 0, i, b.Vx);
                b.Vy = fold_x(f.bc, 1, i, b.Vy);
            }
            b.ie = at.ld(f.ieta, ja, inV);
            b.ieL = __shfl_up_sync(FULL, b.ie, 1);
        }
        if (bstep) {
            // row jb+1's velocities and vertex from A, row jb's cells from A
            cb.Vx = qVx;
            cb.Vy = qVy;
            cb.txy = qT2;
            cb.P = qC2.P;
            cb.txx = qC2.txx;
            cb.tyy = qC2.tyy;
            const MStep<T> ob = x2_step(f, s, b, cb, oa.vx, oa.vy, i, jb, e0, e1, xb, yb, ylo, yhi);
            if (own) {
                if (jb >= js) {
                    at.st(f.P_out, jb, ob.c.P);
                    at.st(f.txx_out, jb, ob.c.txx);
                    at.st(f.tyy_out, jb, ob.c.tyy);
                    if (jb + 1 <= je) at.st(f.txy_out, jb + 1, ob.tn);
                    if (WRITE_RES) {
                        at.st(f.divV, jb, ob.c.dvP);
                        at.st(f.rVx, jb, ob.rx);
                        at.st(f.rVy, jb, ob.ry);
                    }
                    at.st(f.Vx_out, jb, ob.vx);
                    at.st(f.Vy_out, jb, ob.vy);
                } else {
                    at.st(f.txy_out, js, ob.tn);  // vertex row js, computed by B's first row
                }
            }
        }
        qC2 = qC1;
        qC1 = oa.c;
        qT2 = qT1;
        qT1 = oa.tn;
        qVx = oa.vx;
        qVy = oa.vy;
        if (more) cur = nxt;
    }
}

// The arrays of a fused view, for host-side checks.
template <class T>
inline void fused_arrays(const Fused2D<T>& f, const DF<T>* out[22]) {
    const DF<T>* all[22] = {&f.Vx_in, &f.Vy_in, &f.Vx_out, &f.Vy_out, &f.txx_in, &f.tyy_in, &f.txy_in, &f.txx_out,
                            &f.tyy_out, &f.txy_out, &f.P_in, &f.P_out, &f.txx_o, &f.tyy_o, &f.txy_o, &f.ieta,
                            &f.fP, &f.rhox, &f.rhoy, &f.divV, &f.rVx, &f.rVy};
    for (int k = 0; k < 22; ++k) out[k] = all[k];
}

// True when every element offset i + j*s1 the marching kernel forms (i, j in [-1, e+1]) fits
// in a 32-bit int for all of f's arrays.
template <class T>
inline bool march_fits_int(const Fused2D<T>& f, int e0, int e1) {
    const DF<T>* all[22];
    fused_arrays(f, all);
    const long lim = 2147483647L;
    for (const DF<T>* d : all) {
        const long s1 = d->s1 < 0 ? -d->s1 : d->s1;
        if ((long)e0 + 1 + ((long)e1 + 1) * s1 > lim) return false;
    }
    return true;
}

// The row stride shared by every present array of f, or 0 when they differ.
template <class T>
inline long march_uniform_stride(const Fused2D<T>& f) {
    const DF<T>* all[22];
    fused_arrays(f, all);
    long s1 = 0;
    for (const DF<T>* d : all) {
        if (!d->p) continue;
        if (s1 == 0) s1 = d->s1;
        else if (d->s1 != s1) return 0;
    }
    return s1;
}

// Rows per warp of the marching kernel: the length at which the strips x segments warps fill
// every SM once at the kernel's occupancy (one wave), kept within [8, 32] rows. Shorter
// segments re-read more boundary rows; longer ones leave the memory system fewer warps'
// worth of loads in flight (measured on 1024^2 to 4096^2 grids).
template <class T, class Ix, bool UNI, bool WRITE_RES, int MINB = 1>
inline int march_seg_rows(int num_sms, int nstrip, int rows) {
    static const int blocks_per_sm = [] {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march2d_kernel<T, Ix, UNI, WRITE_RES, MINB>, 128,
                                                          0) != cudaSuccess)
            nb = 0;
        return nb > 0 ? nb : 4;
    }();
    const long capacity = (long)num_sms * blocks_per_sm * 4;
    const long nseg = capacity / nstrip > 1 ? capacity / nstrip : 1;
    const int seg = (int)((rows + nseg - 1) / nseg);
    return seg < 8 ? 8 : (seg > 32 ? 32 : seg);
}

template <class T, class Ix, bool UNI, bool WRITE_RES, int MINB = 1>
inline cudaError_t launch_march2d_ix(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, int num_sms, int seg_rows,
                                     long s1u, cudaStream_t st, bool dep = false) {
    const int e0 = n0 + 1, e1 = n1 + 1;
    const int nstrip = cg_div_up(e0 + 1, 30);
    if (seg_rows <= 0) seg_rows = march_seg_rows<T, Ix, UNI, WRITE_RES, MINB>(num_sms, nstrip, e1 + 1);
    const int nseg = cg_div_up(e1 + 1, seg_rows);
    const int nwarps = nstrip * nseg;
    return cg_launch(march2d_kernel<T, Ix, UNI, WRITE_RES, MINB>, dim3(cg_div_up(nwarps, 4)), dim3(128), 0, st, dep, f,
                     s, e0, e1, nstrip, nwarps, seg_rows, s1u);
}

// Launch of the warp-marching kernel over [0, n0+1] x [0, n1+1]; seg_rows <= 0 picks the
// segment length from the occupancy; dep = true makes it a dependent launch (cg_launch).
template <class T, bool WRITE_RES>
inline cudaError_t launch_march2d(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, int num_sms, int seg_rows,
                                  cudaStream_t st, bool dep = false) {
    const long s1u = march_uniform_stride(f);
    // FP32 with one shared stride fits in 64 registers without spills: 8 blocks (32 warps) per SM
    constexpr int minb = sizeof(T) == 4 ? 8 : 1;
    if (march_fits_int(f, n0 + 1, n1 + 1)) {
        if (s1u) return launch_march2d_ix<T, int, true, WRITE_RES, minb>(f, s, n0, n1, num_sms, seg_rows, s1u, st, dep);
        return launch_march2d_ix<T, int, false, WRITE_RES>(f, s, n0, n1, num_sms, seg_rows, 0, st, dep);
    }
    if (s1u) return launch_march2d_ix<T, long, true, WRITE_RES>(f, s, n0, n1, num_sms, seg_rows, s1u, st, dep);
    return launch_march2d_ix<T, long, false, WRITE_RES>(f, s, n0, n1, num_sms, seg_rows, 0, st, dep);
}

// Launch of the two-iteration kernel (march2d_x2_kernel) over [0, n0+1] x [0, n1+1]: two PT
// iterations, `in` -> `out`; fold_a: the first iteration reads its velocities through bc!(V).
// Only for views whose arrays share one row stride and whose offsets fit in 32 bits (the
// callers check march_x2_ok). seg_rows <= 0 picks one wave of warps, 8..64 rows per segment.
// MINB: 4 blocks per SM (up to 128 registers, no spills) or 5 (96 registers, 24 bytes spilled).
template <class T, bool WRITE_RES, int MINB>
inline cudaError_t launch_march2d_x2_mb(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, int num_sms, int seg_rows,
                                        bool fold_a, cudaStream_t st, bool dep) {
    auto kern = march2d_x2_kernel<T, int, true, WRITE_RES, MINB>;
    const long s1u = march_uniform_stride(f);
    const int e0 = n0 + 1, e1 = n1 + 1;
    const int nstrip = cg_div_up(e0 + 1, 28);
    if (seg_rows <= 0) {
        static const int bps = [] {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march2d_x2_kernel<T, int, true, WRITE_RES, MINB>, 128,
                                                              0) != cudaSuccess)
                nb = 0;
            return nb > 0 ? nb : 4;
        }();
        const long capacity = (long)num_sms * bps * 4;
        const long nseg = capacity / nstrip > 1 ? capacity / nstrip : 1;
        seg_rows = (int)((e1 + 1 + nseg - 1) / nseg);
        seg_rows = seg_rows < 8 ? 8 : (seg_rows > 64 ? 64 : seg_rows);
    }
    if (seg_rows < 4) seg_rows = 4;  // no y-plane may lie on a stage's first row
    const int nseg = cg_div_up(e1 + 1, seg_rows);
    const int nwarps = nstrip * nseg;
    return cg_launch(kern, dim3(cg_div_up(nwarps, 4)), dim3(128), 0, st, dep, f, s, e0, e1, nstrip, nwarps, seg_rows, s1u,
                     (int)fold_a);
}

// variant 1: 4 blocks per SM; variant 2: 5 blocks per SM (the autotuner's 2D variants)
template <class T, bool WRITE_RES>
inline cudaError_t launch_march2d_x2(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, int num_sms, int seg_rows,
                                     bool fold_a, cudaStream_t st, bool dep = false, int variant = 1) {
    if (variant == 2) return launch_march2d_x2_mb<T, WRITE_RES, 5>(f, s, n0, n1, num_sms, seg_rows, fold_a, st, dep);
    return launch_march2d_x2_mb<T, WRITE_RES, 4>(f, s, n0, n1, num_sms, seg_rows, fold_a, st, dep);
}

// Whether the two-iteration kernel can take a view: one shared row stride, 32-bit offsets,
// CG_MARCH_X2 not set to 0.
template <class T>
inline bool march_x2_ok(const Fused2D<T>& f, int n0, int n1) {
    static const bool on = [] {
        const char* e = std::getenv("CG_MARCH_X2");
        return !(e && e[0] == '0');
    }();
    return on && march_uniform_stride(f) != 0 && march_fits_int(f, n0 + 1, n1 + 1);
}

}  // namespace cgk
