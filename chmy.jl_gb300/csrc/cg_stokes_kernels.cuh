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

// Read-only loads: in the fused kernel the `in` buffers are never written (ping-pong), so
// the non-coherent path is safe and lets loads move ahead of the stores.
template <class T>
__device__ __forceinline__ T ldg(const DF<T>& f, int i, int j) {
    return __ldg(f.ptr(i, j, 0));
}

template <class T>
__device__ __forceinline__ CellIn<T> load_cell(const Fused2D<T>& f, int i, int j) {
    CellIn<T> c;
    c.P = ldg(f.P_in, i, j);
    c.txx = ldg(f.txx_in, i, j);
    c.tyy = ldg(f.tyy_in, i, j);
    c.txo = ldg(f.txx_o, i, j);
    c.tyo = ldg(f.tyy_o, i, j);
    c.fp = f.has_fP ? ldg(f.fP, i, j) : T(0);
    return c;
}

// Asynchronous global -> shared copy of one element (cp.async, Ampere+). `valid` false
// zero-fills the destination without reading (src-size 0; src must still be a valid address).
template <class T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 4 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared-memory layout of the fused kernel (32 x 32 tile).
template <class T>
struct FusedSmem {
    static constexpr int TX = 32, TY = 32;
    static constexpr int HX = TX + 2, HY = TY + 2;  // V, 1/eta from (i0-1, j0-1)
    static constexpr int CX = TX + 1, CY = TY + 1;  // cells from (i0-1, j0-1); vertices from (i0, j0)
    T Vx[HY][HX], Vy[HY][HX], Ie[HY][HX];
    T P[CY][CX], Txx[CY][CX], Tyy[CY][CX], Txo[CY][CX], Tyo[CY][CX], Fp[CY][CX];  // cells (in -> new)
    T Txy[CY][CX], Txyo[CY][CX];                                                  // vertices (in -> new)
};

// Block (32, 8), tile 32 x 32 of launch points. Phase 0 issues every global read of the block
// as asynchronous copies into shared memory (V and 1/eta on 34 x 34, cell and vertex inputs
// on 33 x 33), so all of them are in flight at once; phase 1 computes the new tau/P on the
// cells and vertices the tile's faces read (own plus a one-point halo) in place; phase 2
// updates the velocity of the tile's own faces. The `in` buffers are never written (ping-pong).
template <class T, bool WRITE_RES>
__global__ void __launch_bounds__(256) fused2d_kernel(const Fused2D<T> f, const SP<T> s, int e0, int e1) {
    using S = FusedSmem<T>;
    constexpr int TX = S::TX, TY = S::TY, HX = S::HX, HY = S::HY, CX = S::CX, CY = S::CY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S& sm = *reinterpret_cast<S*>(smem_raw);
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;

    // ---- phase 0: asynchronous staging ----
    for (int t = tid; t < HX * HY; t += 256) {
        const int a = t % HX, b = t / HX;
        const int ii = i0 - 1 + a, jj = j0 - 1 + b;
        const bool ok = ii <= e0 + 1 && jj <= e1 + 1;
        const int ci = ok ? ii : -1, cj = ok ? jj : -1;  // a valid address when zero-filling
        cp_async_elem(&sm.Vx[b][a], f.Vx_in.ptr(ci, cj, 0), ok);
        cp_async_elem(&sm.Vy[b][a], f.Vy_in.ptr(ci, cj, 0), ok);
        cp_async_elem(&sm.Ie[b][a], f.ieta.ptr(ci, cj, 0), ok);
    }
    for (int t = tid; t < CX * CY; t += 256) {
        const int a = t % CX, b = t / CX;
        // cells (i0-1+a, j0-1+b): needed up to the launch range
        {
            const int ii = i0 - 1 + a, jj = j0 - 1 + b;
            const bool ok = ii <= e0 && jj <= e1;
            const int ci = ok ? ii : -1, cj = ok ? jj : -1;
            cp_async_elem(&sm.P[b][a], f.P_in.ptr(ci, cj, 0), ok);
            cp_async_elem(&sm.Txx[b][a], f.txx_in.ptr(ci, cj, 0), ok);
            cp_async_elem(&sm.Tyy[b][a], f.tyy_in.ptr(ci, cj, 0), ok);
            cp_async_elem(&sm.Txo[b][a], f.txx_o.ptr(ci, cj, 0), ok);
            cp_async_elem(&sm.Tyo[b][a], f.tyy_o.ptr(ci, cj, 0), ok);
            if (f.has_fP) cp_async_elem(&sm.Fp[b][a], f.fP.ptr(ci, cj, 0), ok);
        }
        // vertices (i0+a, j0+b): the old value is needed up to n+2
        {
            const int ii = i0 + a, jj = j0 + b;
            const bool okv = ii <= e0 + 1 && jj <= e1 + 1;
            const bool oko = ii <= e0 && jj <= e1;
            cp_async_elem(&sm.Txy[b][a], f.txy_in.ptr(okv ? ii : 0, okv ? jj : 0, 0), okv);
            cp_async_elem(&sm.Txyo[b][a], f.txy_o.ptr(oko ? ii : 0, oko ? jj : 0, 0), oko);
        }
    }
    cp_async_wait_all();
    __syncthreads();

    const T half = T(0.5);
    // ---- phase 1a: new tau_xx, tau_yy, P at cells (i0-1+a, j0-1+b) in place ----
    for (int t = tid; t < CX * CY; t += 256) {
        const int a = t % CX, b = t / CX;
        const int i = i0 - 1 + a, j = j0 - 1 + b;
        if (i > e0 || j > e1 || i < 0 || j < 0) continue;  // beyond: unused; -1: keeps old value
        const T exx = (sm.Vx[b][a + 1] - sm.Vx[b][a]) * s.idx[0];
        const T eyy = (sm.Vy[b + 1][a] - sm.Vy[b][a]) * s.idx[1];
        const T dv = exx + eyy;
        const T dvP = f.has_fP ? dv + sm.Fp[b][a] : dv;
        const T ie = sm.Ie[b][a];
        const T eve = T(1) / (ie + s.inv_Gdt);
        const T p = sm.P[b][a] - dvP * eve * s.dtau_Pr;
        const T t0 = sm.Txx[b][a], o0 = sm.Txo[b][a];
        const T r0 = -(t0 - o0) * s.inv_Gdt - t0 * ie + T(2.0) * (exx - dv * s.third);
        const T t1 = sm.Tyy[b][a], o1 = sm.Tyo[b][a];
        const T r1 = -(t1 - o1) * s.inv_Gdt - t1 * ie + T(2.0) * (eyy - dv * s.third);
        const T nxx = t0 + r0 * eve * s.dtau_r, nyy = t1 + r1 * eve * s.dtau_r;
        sm.Txx[b][a] = nxx;
        sm.Tyy[b][a] = nyy;
        sm.P[b][a] = p;
        if (a >= 1 && b >= 1) {
            f.txx_out(i, j, 0) = nxx;
            f.tyy_out(i, j, 0) = nyy;
            f.P_out(i, j, 0) = p;
            if (WRITE_RES) f.divV(i, j, 0) = dvP;
        }
    }
    // ---- phase 1b: new tau_xy at vertices (i0+a, j0+b) in place (smem (a+1, b+1) of V) ----
    for (int t = tid; t < CX * CY; t += 256) {
        const int a = t % CX, b = t / CX;
        const int i = i0 + a, j = j0 + b;
        if (i > e0 || j > e1) continue;  // beyond: unused; n+2: keeps old value
        const T exy = half * ((sm.Vx[b + 1][a + 1] - sm.Vx[b][a + 1]) * s.idx[1] +
                              (sm.Vy[b + 1][a + 1] - sm.Vy[b + 1][a]) * s.idx[0]);
        const T e00 = sm.Ie[b][a], e10 = sm.Ie[b][a + 1], e01 = sm.Ie[b + 1][a], e11 = sm.Ie[b + 1][a + 1];
        const T lo = fma(half, e10 - e00, e00);
        const T hi = fma(half, e11 - e01, e01);
        const T iev = fma(half, hi - lo, lo);
        const T eve = T(1) / (iev + s.inv_Gdt);
        const T t2 = sm.Txy[b][a], o2 = sm.Txyo[b][a];
        const T r2 = -(t2 - o2) * s.inv_Gdt - t2 * iev + T(2.0) * exy;
        const T tn = t2 + r2 * eve * s.dtau_r;
        sm.Txy[b][a] = tn;
        if (a < TX && b < TY) f.txy_out(i, j, 0) = tn;
    }
    __syncthreads();

    // ---- phase 2: velocity of the tile's own faces ----
    const int a = threadIdx.x;
    const int i = i0 + a;
#pragma unroll
    for (int r = 0; r < TY / 8; ++r) {
        const int b = threadIdx.y + 8 * r;
        const int j = j0 + b;
        if (i > e0 || j > e1) continue;
        T rx = -((sm.P[b + 1][a + 1] - sm.P[b + 1][a]) * s.idx[0]) + (sm.Txx[b + 1][a + 1] - sm.Txx[b + 1][a]) * s.idx[0];
        rx = rx + (sm.Txy[b + 1][a] - sm.Txy[b][a]) * s.idx[1];
        T ry = -((sm.P[b + 1][a + 1] - sm.P[b][a + 1]) * s.idx[1]) + (sm.Tyy[b + 1][a + 1] - sm.Tyy[b][a + 1]) * s.idx[1];
        ry = ry + (sm.Txy[b][a + 1] - sm.Txy[b][a]) * s.idx[0];
        if (f.has_rho) {
            rx = rx - __ldg(f.rhox.ptr(i, j, 0));
            ry = ry - __ldg(f.rhoy.ptr(i, j, 0));
        }
        if (WRITE_RES) {
            f.rVx(i, j, 0) = rx;
            f.rVy(i, j, 0) = ry;
        }
        const T c = sm.Ie[b + 1][a + 1];
        f.Vx_out(i, j, 0) = sm.Vx[b + 1][a + 1] + rx * (s.nu_dtau * (fmin(sm.Ie[b + 1][a], c) + s.inv_Gdt));
        f.Vy_out(i, j, 0) = sm.Vy[b + 1][a + 1] + ry * (s.nu_dtau * (fmin(sm.Ie[b][a + 1], c) + s.inv_Gdt));
    }
}

// Launch helper: grid of 32 x 32 tiles over [0, n+1]^2, dynamic shared memory opted in.
template <class T, bool WRITE_RES>
inline cudaError_t launch_fused2d(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, cudaStream_t st) {
    const size_t smem = sizeof(FusedSmem<T>);
    // opt in to more than 48 KB of dynamic shared memory (host-side, idempotent; each
    // translation unit holds its own copy of the kernel, so it is set on every call)
    cudaError_t e = cudaFuncSetAttribute(fused2d_kernel<T, WRITE_RES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 block(32, 8), grid(cg_div_up(n0 + 2, 32), cg_div_up(n1 + 2, 32));
    fused2d_kernel<T, WRITE_RES><<<grid, block, smem, st>>>(f, s, n0 + 1, n1 + 1);
    return cudaGetLastError();
}

}  // namespace cgk
