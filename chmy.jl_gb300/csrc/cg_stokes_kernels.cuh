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

// ---- fused 2D PT iteration (variable viscosity): update_stress! + update_velocity! -----------
//
// One launch per PT iteration. A block owns a 32 x TY tile of launch points I; it stages V and
// 1/eta with a halo in shared memory, recomputes the new tau/P on the one-cell halo it needs
// (bitwise the same values the owning block computes), then updates the velocity of its own
// faces. Reads come from the `in` buffers and writes go to the `out` buffers (ping-pong), so the
// redundant halo recomputation never sees a neighbour's new values. Points outside Chmy's
// launch range [0, n+1] keep their old values, exactly as in the two-kernel form.
template <class T>
struct Fused2D {
    DF<T> Vx_in, Vy_in, Vx_out, Vy_out;
    DF<T> txx_in, tyy_in, txy_in, txx_out, tyy_out, txy_out, P_in, P_out;
    DF<T> txx_o, tyy_o, txy_o, ieta, fP, rhox, rhoy, divV, rVx, rVy;
    int has_fP, has_rho;
};

// Cell update of the fused kernel: new tau_xx, tau_yy, P at cell (i, j) whose smem coordinates
// in the staged V / 1/eta tile are (a, b) (the staged tile starts at (i0-1, j0-1)).
template <class T>
struct CellIn {
    T P, txx, tyy, txo, tyo, fp;
};

template <class T, int HX>
__device__ __forceinline__ void fused_cell(const Fused2D<T>& f, const SP<T>& s, const T (*sVx)[HX],
                                           const T (*sVy)[HX], const T (*sIe)[HX], int a, int b, const CellIn<T>& c,
                                           T& nxx, T& nyy, T& nP, T& dvP_out) {
    const T exx = (sVx[b][a + 1] - sVx[b][a]) * s.idx[0];
    const T eyy = (sVy[b + 1][a] - sVy[b][a]) * s.idx[1];
    const T dv = exx + eyy;
    const T dvP = f.has_fP ? dv + c.fp : dv;
    const T ie = sIe[b][a];
    const T eve = T(1) / (ie + s.inv_Gdt);
    nP = c.P - dvP * eve * s.dtau_Pr;
    const T r0 = -(c.txx - c.txo) * s.inv_Gdt - c.txx * ie + T(2.0) * (exx - dv * s.third);
    const T r1 = -(c.tyy - c.tyo) * s.inv_Gdt - c.tyy * ie + T(2.0) * (eyy - dv * s.third);
    nxx = c.txx + r0 * eve * s.dtau_r;
    nyy = c.tyy + r1 * eve * s.dtau_r;
    dvP_out = dvP;
}

// Vertex update: new tau_xy at vertex (i, j) = staged smem coordinates (a+1, b+1).
template <class T, int HX>
__device__ __forceinline__ T fused_vertex(const SP<T>& s, const T (*sVx)[HX], const T (*sVy)[HX],
                                          const T (*sIe)[HX], int a, int b, T t2, T o2) {
    const T half = T(0.5);
    const T exy = half * ((sVx[b + 1][a + 1] - sVx[b][a + 1]) * s.idx[1] + (sVy[b + 1][a + 1] - sVy[b + 1][a]) * s.idx[0]);
    const T e00 = sIe[b][a], e10 = sIe[b][a + 1], e01 = sIe[b + 1][a], e11 = sIe[b + 1][a + 1];
    const T lo = fma(half, e10 - e00, e00);
    const T hi = fma(half, e11 - e01, e01);
    const T iev = fma(half, hi - lo, lo);
    const T eve = T(1) / (iev + s.inv_Gdt);
    const T r2 = -(t2 - o2) * s.inv_Gdt - t2 * iev + T(2.0) * exy;
    return t2 + r2 * eve * s.dtau_r;
}

template <class T>
__device__ __forceinline__ CellIn<T> load_cell(const Fused2D<T>& f, int i, int j) {
    CellIn<T> c;
    c.P = f.P_in(i, j, 0);
    c.txx = f.txx_in(i, j, 0);
    c.tyy = f.tyy_in(i, j, 0);
    c.txo = f.txx_o(i, j, 0);
    c.tyo = f.tyy_o(i, j, 0);
    c.fp = f.has_fP ? f.fP(i, j, 0) : T(0);
    return c;
}

// Block (32, 8), tile 32 x 32 of launch points; every global load of a thread is issued before
// the first barrier (own cells, vertices and faces in registers, V and 1/eta staged in shared
// memory), so that ~50 loads per thread are in flight at once.
template <class T, bool WRITE_RES>
__global__ void __launch_bounds__(256, 2) fused2d_kernel(const Fused2D<T> f, const SP<T> s, int e0, int e1) {
    constexpr int TX = 32, R = 4, TY = 8 * R;
    constexpr int HX = TX + 2, HY = TY + 2;  // V, 1/eta staged from (i0-1, j0-1)
    constexpr int CX = TX + 1, CY = TY + 1;  // new cells from (i0-1, j0-1); new vertices from (i0, j0)
    __shared__ T sVx[HY][HX], sVy[HY][HX], sIe[HY][HX];
    __shared__ T sTxx[CY][CX], sTyy[CY][CX], sP[CY][CX], sTxy[CY][CX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int i = i0 + tx;

    // ---- loads: own cells / vertices / faces at (i, j0 + ty + 8r) ----
    CellIn<T> cin[R];
    T vxy[R], vxo[R], rhx[R], rhy[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + ty + 8 * r;
        const bool cell_in = i <= e0 && j <= e1;
        const bool vert_in = i <= e0 + 1 && j <= e1 + 1;
        if (cell_in) cin[r] = load_cell(f, i, j);
        vxy[r] = vert_in ? f.txy_in(i, j, 0) : T(0);
        vxo[r] = cell_in ? f.txy_o(i, j, 0) : T(0);
        rhx[r] = (cell_in && f.has_rho) ? f.rhox(i, j, 0) : T(0);
        rhy[r] = (cell_in && f.has_rho) ? f.rhoy(i, j, 0) : T(0);
    }
    // halo items: warp 0 cell row j0-1 (a = tx, and a = 32 for lane 0); warp 1 cell column i0-1;
    // warp 2 vertex row j0+32; warp 3 vertex column i0+32 (and the corner for lane 0)
    CellIn<T> hc[2];
    T hv[2], hvo[2];
    int hi_[2], hj_[2], hn = 0;
    if (ty == 0) {
        hi_[0] = i0 - 1 + tx;
        hj_[0] = j0 - 1;
        hi_[1] = i0 - 1 + 32;
        hj_[1] = j0 - 1;
        hn = tx == 0 ? 2 : 1;
    } else if (ty == 1) {
        hi_[0] = i0 - 1;
        hj_[0] = j0 + tx;
        hn = 1;
    } else if (ty == 2) {
        hi_[0] = i0 + tx;
        hj_[0] = j0 + 32;
        hn = 1;
    } else if (ty == 3) {
        hi_[0] = i0 + 32;
        hj_[0] = j0 + tx;
        hi_[1] = i0 + 32;
        hj_[1] = j0 + 32;
        hn = tx == 0 ? 2 : 1;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (h >= hn) break;
        const int hi = hi_[h], hj = hj_[h];
        if (ty <= 1) {
            if (hi <= e0 && hj <= e1) hc[h] = load_cell(f, hi, hj);
        } else {
            hv[h] = (hi <= e0 + 1 && hj <= e1 + 1) ? f.txy_in(hi, hj, 0) : T(0);
            hvo[h] = (hi <= e0 && hj <= e1) ? f.txy_o(hi, hj, 0) : T(0);
        }
    }
    // staged V and 1/eta over logical [i0-1, i0+32] x [j0-1, j0+32], clipped to [-1, n+2]
#pragma unroll
    for (int bb = 0; bb < (HY + 7) / 8; ++bb) {
        const int b = ty + 8 * bb;
        if (b >= HY) break;
#pragma unroll
        for (int aa = 0; aa < 2; ++aa) {
            const int a = tx + 32 * aa;
            if (a >= HX) break;
            const int ii = i0 - 1 + a, jj = j0 - 1 + b;
            const bool ok = ii <= e0 + 1 && jj <= e1 + 1;
            sVx[b][a] = ok ? f.Vx_in(ii, jj, 0) : T(0);
            sVy[b][a] = ok ? f.Vy_in(ii, jj, 0) : T(0);
            sIe[b][a] = ok ? f.ieta(ii, jj, 0) : T(0);
        }
    }
    __syncthreads();

    // ---- phase 1: new tau/P at own cells and vertices, then the halo ones ----
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + ty + 8 * r;
        const int a = tx + 1, b = ty + 1 + 8 * r;  // cell smem coords
        if (i <= e0 && j <= e1) {
            T nxx, nyy, nP, dvP;
            fused_cell<T, HX>(f, s, sVx, sVy, sIe, a, b, cin[r], nxx, nyy, nP, dvP);
            sTxx[b][a] = nxx;
            sTyy[b][a] = nyy;
            sP[b][a] = nP;
            f.txx_out(i, j, 0) = nxx;
            f.tyy_out(i, j, 0) = nyy;
            f.P_out(i, j, 0) = nP;
            if (WRITE_RES) f.divV(i, j, 0) = dvP;
        }
        // own vertex (tx, ty + 8r): in range -> new value; the vertex n+2 -> old value
        const int va = tx, vb = ty + 8 * r;
        if (i <= e0 + 1 && j <= e1 + 1) {
            if (i <= e0 && j <= e1) {
                const T tn = fused_vertex<T, HX>(s, sVx, sVy, sIe, va, vb, vxy[r], vxo[r]);
                sTxy[vb][va] = tn;
                f.txy_out(i, j, 0) = tn;
            } else {
                sTxy[vb][va] = vxy[r];
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (h >= hn) break;
        const int hi = hi_[h], hj = hj_[h];
        if (ty <= 1) {
            const int a = hi - (i0 - 1), b = hj - (j0 - 1);
            if (hi > e0 || hj > e1) continue;
            if (hi < 0 || hj < 0) {  // outside the launch range: old values
                sTxx[b][a] = hc[h].txx;
                sTyy[b][a] = hc[h].tyy;
                sP[b][a] = hc[h].P;
            } else {
                T nxx, nyy, nP, dvP;
                fused_cell<T, HX>(f, s, sVx, sVy, sIe, a, b, hc[h], nxx, nyy, nP, dvP);
                sTxx[b][a] = nxx;
                sTyy[b][a] = nyy;
                sP[b][a] = nP;
            }
        } else {
            const int a = hi - i0, b = hj - j0;
            if (hi > e0 + 1 || hj > e1 + 1) continue;
            if (hi > e0 || hj > e1) sTxy[b][a] = hv[h];
            else sTxy[b][a] = fused_vertex<T, HX>(s, sVx, sVy, sIe, a, b, hv[h], hvo[h]);
        }
    }
    __syncthreads();

    // ---- phase 2: velocity of the tile's own faces ----
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int a = tx, b = ty + 8 * r;
        const int j = j0 + b;
        if (i > e0 || j > e1) continue;
        // cells: smem (a+1, b+1) = (i, j); vertices: smem (a, b) = (i, j)
        T rx = -((sP[b + 1][a + 1] - sP[b + 1][a]) * s.idx[0]) + (sTxx[b + 1][a + 1] - sTxx[b + 1][a]) * s.idx[0];
        rx = rx + (sTxy[b + 1][a] - sTxy[b][a]) * s.idx[1];
        T ry = -((sP[b + 1][a + 1] - sP[b][a + 1]) * s.idx[1]) + (sTyy[b + 1][a + 1] - sTyy[b][a + 1]) * s.idx[1];
        ry = ry + (sTxy[b][a + 1] - sTxy[b][a]) * s.idx[0];
        if (f.has_rho) {
            rx = rx - rhx[r];
            ry = ry - rhy[r];
        }
        if (WRITE_RES) {
            f.rVx(i, j, 0) = rx;
            f.rVy(i, j, 0) = ry;
        }
        const T c = sIe[b + 1][a + 1];
        f.Vx_out(i, j, 0) = sVx[b + 1][a + 1] + rx * (s.nu_dtau * (fmin(sIe[b + 1][a], c) + s.inv_Gdt));
        f.Vy_out(i, j, 0) = sVy[b + 1][a + 1] + ry * (s.nu_dtau * (fmin(sIe[b][a + 1], c) + s.inv_Gdt));
    }
}

}  // namespace cgk
