// cg_march3d.cuh — fused 3D VE Stokes PT iteration (update_stress! + update_velocity!,
// examples/stokes_3d_inc_ve_T.jl:23-57, variable-viscosity form) as a z-marching kernel.
#pragma once

#include "cg_stokes_kernels.cuh"

namespace cgk {

// Ping-pong views of one fused 3D iteration: the `in` buffers are read, the `out` buffers
// written. Tensor order (xx, yy, zz, xy, xz, yz).
template <class T>
struct Fused3D {
    DF<T> V_in[3], V_out[3], tau_in[6], tau_out[6], P_in, P_out;
    DF<T> tau_o[6], ieta, fP, rho[3], divV, rV[3];
    int has_fP, has_rho[3];
};

// Element offsets of lane column i, row j: UNI when every array shares the strides s1u, s2u.
template <class T, class Ix, bool UNI>
struct MAt3 {
    int i, j;
    Ix s1u, s2u;
    __device__ __forceinline__ Ix off(const DF<T>& f, int k) const {
        return (Ix)i + (Ix)j * (UNI ? s1u : (Ix)f.s1) + (Ix)k * (UNI ? s2u : (Ix)f.s2);
    }
    __device__ __forceinline__ T ld(const DF<T>& f, int k, bool ok) const { return ok ? __ldg(f.p + off(f, k)) : T(0); }
    __device__ __forceinline__ void st(const DF<T>& f, int k, T v) const { f.p[off(f, k)] = v; }
};

// Inputs of z-step k at one (i, j): plane k+1 of V, 1/eta and the xz/yz shear inputs, plane k
// of the cell and xy inputs.
template <class T>
struct M3Row {
    T vx, vy, vz, ie, txz, txzo, tyz, tyzo;                                 // plane k+1
    T P, txx, tyy, tzz, txo, tyo, tzo, txy, txyo, fp, rhox, rhoy, rhoz;  // plane k
};

// Which inputs a warp reads: owned rows read all; the lower halo row only what the new P and
// tau_yy of its cells need; the upper halo row only what its new tau_xy and tau_yz need.
struct M3Need {
    bool cell_p, cell_d, xy, yz, xz, rho;  // P/tau_yy/tau_yy_old/fP; other diagonals; xy; yz; xz; rho g
};

template <class T, class Ix, bool UNI>
__device__ __forceinline__ M3Row<T> m3_load(const Fused3D<T>& f, const MAt3<T, Ix, UNI>& at, int k, int e2, bool inV,
                                            bool inC, const M3Need& nd) {
    M3Row<T> r;
    const int kn = k + 1;
    const bool vn = inV && kn <= e2 + 1;  // V, 1/eta, shear inputs (readable to n+2)
    const bool cn = inC && kn <= e2;      // shear olds (needed up to the launch range)
    r.vx = at.ld(f.V_in[0], kn, vn);
    r.vy = at.ld(f.V_in[1], kn, vn);
    r.vz = at.ld(f.V_in[2], kn, vn);
    r.ie = at.ld(f.ieta, kn, vn);
    r.txz = at.ld(f.tau_in[4], kn, vn && nd.xz);
    r.txzo = at.ld(f.tau_o[4], kn, cn && nd.xz);
    r.tyz = at.ld(f.tau_in[5], kn, vn && nd.yz);
    r.tyzo = at.ld(f.tau_o[5], kn, cn && nd.yz);
    const bool c = inC && k <= e2;
    const bool v = inV && k <= e2;
    r.P = at.ld(f.P_in, k, c && nd.cell_p);
    r.tyy = at.ld(f.tau_in[1], k, c && nd.cell_p);
    r.tyo = at.ld(f.tau_o[1], k, c && nd.cell_p);
    r.fp = f.has_fP ? at.ld(f.fP, k, c && nd.cell_p) : T(0);
    r.txx = at.ld(f.tau_in[0], k, c && nd.cell_d);
    r.tzz = at.ld(f.tau_in[2], k, c && nd.cell_d);
    r.txo = at.ld(f.tau_o[0], k, c && nd.cell_d);
    r.tzo = at.ld(f.tau_o[2], k, c && nd.cell_d);
    r.txy = at.ld(f.tau_in[3], k, v && nd.xy);
    r.txyo = at.ld(f.tau_o[3], k, c && nd.xy);
    r.rhox = f.has_rho[0] ? at.ld(f.rho[0], k, c && nd.rho) : T(0);
    r.rhoy = f.has_rho[1] ? at.ld(f.rho[1], k, c && nd.rho) : T(0);
    r.rhoz = f.has_rho[2] ? at.ld(f.rho[2], k, c && nd.rho) : T(0);
    return r;
}

// ---- point arithmetic (V: the value type, S: its scalar parameters' type) -------------------
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ double vneg(double a) { return -a; }
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double vmin(double a, double b) { return fmin(a, b); }
template <class V, class S>
__device__ __forceinline__ V bcast(S x) {
    return x;
}

// -(t - t_old) * inv_Gdt - t * ieta + 2 * e: the VE stress residual, left to right.
template <class V, class S>
__device__ __forceinline__ V m3_res(const SP<S>& s, V t, V to, V ie, V e) {
    return radd(rsub(rmul(vneg(rsub(t, to)), s.inv_Gdt), rmul(t, ie)), rmul(e, S(2.0)));
}

// New shear stress on an (a, b) edge from its strain rate and the four cells' 1/eta around it
// (e00 = both indices decremented, e10 = b decremented, e01 = a decremented, e11 = none),
// interpolated with the Linear rule, a innermost.
template <class V, class S>
__device__ __forceinline__ V m3_shear(const SP<S>& s, V e, V e00, V e10, V e01, V e11, V t, V to) {
    const V half = bcast<V>(S(0.5));
    const V lo = rfma(half, rsub(e10, e00), e00);
    const V hi = rfma(half, rsub(e11, e01), e01);
    const V iev = rfma(half, rsub(hi, lo), lo);
    const V eve = rrcp(radd(iev, s.inv_Gdt));
    return radd(t, rmul(rmul(m3_res(s, t, to, iev, e), eve), s.dtau_r));
}

// 0.5 * (d_b(V_a) + d_a(V_b)) with each derivative (right - left) * inverse spacing.
template <class V, class S>
__device__ __forceinline__ V m3_rate(V a1, V a0, S ia, V b1, V b0, S ib) {
    return rmul(radd(rmul(rsub(a1, a0), ia), rmul(rsub(b1, b0), ib)), S(0.5));
}

template <class V>
struct Cell3 {
    V P, txx, tyy, tzz, dvP;
};

// New P and diagonal stresses at a cell from its velocity differences (update_stress!).
template <class V, class S>
__device__ __forceinline__ Cell3<V> m3_cell(const SP<S>& s, bool has_fP, V dvx, V dvy, V dvz, V ie, V P, V txx, V txo,
                                            V tyy, V tyo, V tzz, V tzo, V fp) {
    const V exx = rmul(dvx, s.idx[0]);
    const V eyy = rmul(dvy, s.idx[1]);
    const V ezz = rmul(dvz, s.idx[2]);
    const V dv = radd(radd(exx, eyy), ezz);
    const V dvt = rmul(dv, s.third);
    const V eve = rrcp(radd(ie, s.inv_Gdt));
    Cell3<V> c;
    c.dvP = has_fP ? radd(dv, fp) : dv;
    c.P = rsub(P, rmul(rmul(c.dvP, eve), s.dtau_Pr));
    c.txx = radd(txx, rmul(rmul(m3_res(s, txx, txo, ie, rsub(exx, dvt)), eve), s.dtau_r));
    c.tyy = radd(tyy, rmul(rmul(m3_res(s, tyy, tyo, ie, rsub(eyy, dvt)), eve), s.dtau_r));
    c.tzz = radd(tzz, rmul(rmul(m3_res(s, tzz, tzo, ie, rsub(ezz, dvt)), eve), s.dtau_r));
    return c;
}

// Values exchanged between the y-rows of a block through shared memory each z-step.
template <class T, int NW>
struct M3Smem {
    T vx[NW][32], vy[NW][32], vz[NW][32], ie[NW][32];  // old values (A)
    T P[NW][32], tyy[NW][32], txy[NW][32], tyz[NW][32];  // new values (B)
};

// A block is NW warps. Warp w holds row j = j0 - 1 + w of a tile of 30 x (NW - 2) owned
// (i, j) columns. Lane l holds column i = i0 - 1 + l, so lanes 0 and 31 and warps 0 and NW-1
// are one-point halos. The block marches up the planes k = ks .. ke of its z segment. Each
// z-step: (A) every row stores the old values its y-neighbours need and the block syncs; the
// rows compute the new cells and tau_xy at plane k and tau_xz, tau_yz at plane k+1; (B) they
// store the new values the neighbours need and the block syncs; the owned rows update the
// velocity at plane k. x-neighbours come from shuffles, z-neighbours from registers. The
// arithmetic rounds every operation as the CPU oracle does (see radd/rmul).
template <class T, class Ix, bool UNI, bool WRITE_RES, int NW, int MINB, bool PREF = true>
__global__ void __launch_bounds__(32 * NW, MINB)
    march3d_kernel(const Fused3D<T> f, const SP<T> s, int e0, int e1, int e2, int nstrip, int ntile_y, int seg_len,
                   long s1u, long s2u) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ M3Smem<T, NW> sm;
    cg_dep_wait();
    cg_dep_release();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int strip = b % nstrip, ty = (b / nstrip) % ntile_y, seg = b / (nstrip * ntile_y);
    const int ks = seg * seg_len;
    if (ks > e2) return;  // whole block
    const int ke = min(ks + seg_len - 1, e2);
    const int i = strip * 30 - 1 + lane;
    const int j = ty * (NW - 2) - 1 + w;
    const bool lo = w == 0, hi = w == NW - 1;
    const bool own = !lo && !hi && lane >= 1 && lane <= 30 && i <= e0 && j <= e1;
    const bool inV = i <= e0 + 1 && j <= e1 + 1;  // V, 1/eta, shear inputs readable
    const bool inC = i <= e0 && j <= e1;          // cell inputs, shear olds readable
    const bool oldcell_ij = i < 0 || j < 0;       // column or row -1 keeps its old cells
    M3Need nd;
    nd.cell_p = !hi;
    nd.cell_d = !lo && !hi;
    nd.xy = !lo;
    nd.yz = !lo;
    nd.xz = !lo && !hi;
    nd.rho = !lo && !hi;
    const MAt3<T, Ix, UNI> at{i, j, (Ix)s1u, (Ix)s2u};
    const int wu = w + 1 < NW ? w + 1 : NW - 1, wd = w > 0 ? w - 1 : 0;  // in-bounds neighbours
    const int ll = lane > 0 ? lane - 1 : 0;

    // ---- prologue: new P, tau_zz at plane ks-1; new tau_xz, tau_yz at plane ks ----
    T vx_c, vy_c, vz_c, ie_c, ie_p, ieL_c, ieD_c, ieDL_c, Pn_p, tzzn_p, txz_c, tyz_c;
    {
        const int kp = ks - 1;  // >= -1
        const T vxp = at.ld(f.V_in[0], kp, inV), vyp = at.ld(f.V_in[1], kp, inV), vzp = at.ld(f.V_in[2], kp, inV);
        const T iep = at.ld(f.ieta, kp, inV);
        const T pp = at.ld(f.P_in, kp, inC && !hi), tzp = at.ld(f.tau_in[2], kp, inC && !hi);
        const T tzop = at.ld(f.tau_o[2], kp, inC && !hi);
        const T fpp = f.has_fP ? at.ld(f.fP, kp, inC && !hi) : T(0);
        vx_c = at.ld(f.V_in[0], ks, inV);
        vy_c = at.ld(f.V_in[1], ks, inV);
        vz_c = at.ld(f.V_in[2], ks, inV);
        ie_c = at.ld(f.ieta, ks, inV);
        const T txz0 = at.ld(f.tau_in[4], ks, inV && nd.xz), txzo0 = at.ld(f.tau_o[4], ks, inC && nd.xz);
        const T tyz0 = at.ld(f.tau_in[5], ks, inV && nd.yz), tyzo0 = at.ld(f.tau_o[5], ks, inC && nd.yz);
        sm.vx[w][lane] = iep;  // 1/eta at plane ks-1
        sm.vy[w][lane] = vyp;
        sm.vz[w][lane] = vz_c;
        sm.ie[w][lane] = ie_c;
        __syncthreads();
        const T vyUp = sm.vy[wu][lane];   // Vy(i, j+1, ks-1)
        const T iepD = sm.vx[wd][lane];   // 1/eta(i, j-1, ks-1)
        const T vzD = sm.vz[wd][lane];    // Vz(i, j-1, ks)
        ieD_c = sm.ie[wd][lane];          // 1/eta(i, j-1, ks)
        ieDL_c = sm.ie[wd][ll];           // 1/eta(i-1, j-1, ks)
        const T vxpR = __shfl_down_sync(FULL, vxp, 1);
        const Cell3<T> cp = m3_cell(s, f.has_fP != 0, rsub(vxpR, vxp), rsub(vyUp, vyp), rsub(vz_c, vzp), iep, pp, T(0),
                                    T(0), T(0), T(0), tzp, tzop, fpp);
        const bool keep = kp < 0 || oldcell_ij;
        Pn_p = keep ? pp : cp.P;
        tzzn_p = keep ? tzp : cp.tzz;
        const T vzL = __shfl_up_sync(FULL, vz_c, 1);
        const T iepL = __shfl_up_sync(FULL, iep, 1);
        ieL_c = __shfl_up_sync(FULL, ie_c, 1);
        // tau_xz at (i, j, ks): a = x, b = z
        txz_c = (i > e0) ? txz0
                         : m3_shear(s, m3_rate(vx_c, vxp, s.idx[2], vz_c, vzL, s.idx[0]), iepL, iep, ieL_c, ie_c, txz0,
                                    txzo0);
        // tau_yz at (i, j, ks): a = y, b = z
        tyz_c = (j > e1) ? tyz0
                         : m3_shear(s, m3_rate(vy_c, vyp, s.idx[2], vz_c, vzD, s.idx[1]), iepD, iep, ieD_c, ie_c, tyz0,
                                    tyzo0);
        if (own) {
            at.st(f.tau_out[4], ks, txz_c);
            at.st(f.tau_out[5], ks, tyz_c);
        }
        ie_p = iep;
        __syncthreads();  // the prologue's reads of A before the first step's writes
    }

    // PREF: the next step's loads are issued before the current step is computed
    M3Row<T> cur;
    if (PREF) cur = m3_load(f, at, ks, e2, inV, inC, nd);
    for (int k = ks; k <= ke; ++k) {
        M3Row<T> nxt;
        if (PREF) {
            if (k < ke) nxt = m3_load(f, at, k + 1, e2, inV, inC, nd);
        } else {
            cur = m3_load(f, at, k, e2, inV, inC, nd);
        }
        // (A) old values for the y-neighbours
        sm.vx[w][lane] = vx_c;
        sm.vy[w][lane] = vy_c;
        sm.vz[w][lane] = cur.vz;
        sm.ie[w][lane] = cur.ie;
        __syncthreads();
        const T vyU = sm.vy[wu][lane];    // Vy(i, j+1, k)
        const T vxD = sm.vx[wd][lane];    // Vx(i, j-1, k)
        const T vzDn = sm.vz[wd][lane];   // Vz(i, j-1, k+1)
        const T ieDn = sm.ie[wd][lane];   // 1/eta(i, j-1, k+1)
        const T ieDLn = sm.ie[wd][ll];    // 1/eta(i-1, j-1, k+1)
        // new cell (i, j, k)
        const T vxR = __shfl_down_sync(FULL, vx_c, 1);
        Cell3<T> c = m3_cell(s, f.has_fP != 0, rsub(vxR, vx_c), rsub(vyU, vy_c), rsub(cur.vz, vz_c), ie_c, cur.P,
                             cur.txx, cur.txo, cur.tyy, cur.tyo, cur.tzz, cur.tzo, cur.fp);
        if (oldcell_ij) {
            c.P = cur.P;
            c.txx = cur.txx;
            c.tyy = cur.tyy;
            c.tzz = cur.tzz;
        }
        // new tau_xy at (i, j, k): a = x, b = y
        const T vyL = __shfl_up_sync(FULL, vy_c, 1);
        const T txyn = (i > e0 || j > e1)
                           ? cur.txy
                           : m3_shear(s, m3_rate(vx_c, vxD, s.idx[1], vy_c, vyL, s.idx[0]), ieDL_c, ieD_c, ieL_c, ie_c,
                                      cur.txy, cur.txyo);
        // new tau_xz, tau_yz at (i, j, k+1)
        const T vzLn = __shfl_up_sync(FULL, cur.vz, 1);
        const T ieLn = __shfl_up_sync(FULL, cur.ie, 1);
        const T txzn = (i > e0 || k + 1 > e2)
                           ? cur.txz
                           : m3_shear(s, m3_rate(cur.vx, vx_c, s.idx[2], cur.vz, vzLn, s.idx[0]), ieL_c, ie_c, ieLn,
                                      cur.ie, cur.txz, cur.txzo);
        const T tyzn = (j > e1 || k + 1 > e2)
                           ? cur.tyz
                           : m3_shear(s, m3_rate(cur.vy, vy_c, s.idx[2], cur.vz, vzDn, s.idx[1]), ieD_c, ie_c, ieDn,
                                      cur.ie, cur.tyz, cur.tyzo);
        // (B) new values for the y-neighbours
        sm.P[w][lane] = c.P;
        sm.tyy[w][lane] = c.tyy;
        sm.txy[w][lane] = txyn;
        sm.tyz[w][lane] = tyz_c;
        __syncthreads();
        const T PD = sm.P[wd][lane];       // P(i, j-1, k)
        const T tyyD = sm.tyy[wd][lane];   // tau_yy(i, j-1, k)
        const T txyU = sm.txy[wu][lane];   // tau_xy(i, j+1, k)
        const T tyzU = sm.tyz[wu][lane];   // tau_yz(i, j+1, k)
        // velocity (i, j, k): r_V.d = -d_d(P) + d_d(tau_dd) + the off-diagonal terms in the
        // order x: (xy, xz), y: (xy, yz), z: (xz, yz), then - rho g
        const T PL = __shfl_up_sync(FULL, c.P, 1);
        const T txxL = __shfl_up_sync(FULL, c.txx, 1);
        const T txyR = __shfl_down_sync(FULL, txyn, 1);
        const T txzR = __shfl_down_sync(FULL, txz_c, 1);
        if (own) {
            T rx = radd(-rmul(rsub(c.P, PL), s.idx[0]), rmul(rsub(c.txx, txxL), s.idx[0]));
            rx = radd(rx, rmul(rsub(txyU, txyn), s.idx[1]));
            rx = radd(rx, rmul(rsub(txzn, txz_c), s.idx[2]));
            T ry = radd(-rmul(rsub(c.P, PD), s.idx[1]), rmul(rsub(c.tyy, tyyD), s.idx[1]));
            ry = radd(ry, rmul(rsub(txyR, txyn), s.idx[0]));
            ry = radd(ry, rmul(rsub(tyzn, tyz_c), s.idx[2]));
            T rz = radd(-rmul(rsub(c.P, Pn_p), s.idx[2]), rmul(rsub(c.tzz, tzzn_p), s.idx[2]));
            rz = radd(rz, rmul(rsub(txzR, txz_c), s.idx[0]));
            rz = radd(rz, rmul(rsub(tyzU, tyz_c), s.idx[1]));
            if (f.has_rho[0]) rx = rsub(rx, cur.rhox);
            if (f.has_rho[1]) ry = rsub(ry, cur.rhoy);
            if (f.has_rho[2]) rz = rsub(rz, cur.rhoz);
            at.st(f.P_out, k, c.P);
            at.st(f.tau_out[0], k, c.txx);
            at.st(f.tau_out[1], k, c.tyy);
            at.st(f.tau_out[2], k, c.tzz);
            at.st(f.tau_out[3], k, txyn);
            if (k + 1 <= ke) {
                at.st(f.tau_out[4], k + 1, txzn);
                at.st(f.tau_out[5], k + 1, tyzn);
            }
            if (WRITE_RES) {
                at.st(f.divV, k, c.dvP);
                at.st(f.rV[0], k, rx);
                at.st(f.rV[1], k, ry);
                at.st(f.rV[2], k, rz);
            }
            at.st(f.V_out[0], k, radd(vx_c, rmul(rx, rmul(s.nu_dtau, radd(fmin(ieL_c, ie_c), s.inv_Gdt)))));
            at.st(f.V_out[1], k, radd(vy_c, rmul(ry, rmul(s.nu_dtau, radd(fmin(ieD_c, ie_c), s.inv_Gdt)))));
            at.st(f.V_out[2], k, radd(vz_c, rmul(rz, rmul(s.nu_dtau, radd(fmin(ie_p, ie_c), s.inv_Gdt)))));
        }
        // advance one plane
        vx_c = cur.vx;
        vy_c = cur.vy;
        vz_c = cur.vz;
        ie_p = ie_c;
        ie_c = cur.ie;
        ieL_c = ieLn;
        ieD_c = ieDn;
        ieDL_c = ieDLn;
        Pn_p = c.P;
        tzzn_p = c.tzz;
        txz_c = txzn;
        tyz_c = tyzn;
        if (PREF) cur = nxt;
    }
}

// The arrays of a fused 3D view, for host-side checks.
template <class T>
inline int fused3_arrays(const Fused3D<T>& f, const DF<T>* out[40]) {
    int n = 0;
    for (int d = 0; d < 3; ++d) {
        out[n++] = &f.V_in[d];
        out[n++] = &f.V_out[d];
        out[n++] = &f.rho[d];
        out[n++] = &f.rV[d];
    }
    for (int c = 0; c < 6; ++c) {
        out[n++] = &f.tau_in[c];
        out[n++] = &f.tau_out[c];
        out[n++] = &f.tau_o[c];
    }
    out[n++] = &f.P_in;
    out[n++] = &f.P_out;
    out[n++] = &f.ieta;
    out[n++] = &f.fP;
    out[n++] = &f.divV;
    return n;
}

// True when every offset i + j*s1 + k*s2 (indices in [-1, e+1]) fits in a 32-bit int.
template <class T>
inline bool march3_fits_int(const Fused3D<T>& f, int e0, int e1, int e2) {
    const DF<T>* all[40];
    const int n = fused3_arrays(f, all);
    for (int q = 0; q < n; ++q) {
        const long s1 = all[q]->s1 < 0 ? -all[q]->s1 : all[q]->s1, s2 = all[q]->s2 < 0 ? -all[q]->s2 : all[q]->s2;
        if ((long)e0 + 1 + ((long)e1 + 1) * s1 + ((long)e2 + 1) * s2 > 2147483647L) return false;
    }
    return true;
}

// Whether every present array shares the row and plane strides (returned in s1, s2).
template <class T>
inline bool march3_uniform(const Fused3D<T>& f, long* s1, long* s2) {
    const DF<T>* all[40];
    const int n = fused3_arrays(f, all);
    *s1 = 0;
    *s2 = 0;
    for (int q = 0; q < n; ++q) {
        if (!all[q]->p) continue;
        if (*s1 == 0) {
            *s1 = all[q]->s1;
            *s2 = all[q]->s2;
        } else if (all[q]->s1 != *s1 || all[q]->s2 != *s2) {
            return false;
        }
    }
    return *s1 != 0;
}

constexpr int kM3Warps = 8;  // default y-rows per block (owned rows + 2 halo rows)

// Z-segment length: the number of segments whose blocks fill the resident slots best (whole
// waves), with segments of at least 16 planes.
inline int m3_seg_len(long tiles, int planes, long cap) {
    int best = 1;
    double best_eff = 0;
    for (int ns = 1; ns <= 64 && (ns == 1 || planes / ns >= 16); ++ns) {
        const int len = cg_div_up(planes, ns);
        const long items = tiles * cg_div_up(planes, len);
        const long waves = (items + cap - 1) / cap;
        const double eff = (double)items / (double)(waves * cap) * (double)len / (double)(len + 1);
        if (eff > best_eff + 1e-3) {
            best_eff = eff;
            best = ns;
        }
    }
    return cg_div_up(planes, best);
}

template <class T, class Ix, bool UNI, bool WRITE_RES, int MINB, int NW = kM3Warps, bool PREF = true>
inline cudaError_t launch_march3d_ix(const Fused3D<T>& f, const SP<T>& s, int n0, int n1, int n2, int num_sms,
                                     int seg_len, long s1u, long s2u, cudaStream_t st, bool dep = false) {
    const int e0 = n0 + 1, e1 = n1 + 1, e2 = n2 + 1;
    const int nstrip = cg_div_up(e0 + 1, 30), nty = cg_div_up(e1 + 1, NW - 2);
    const long tiles = (long)nstrip * nty;
    if (seg_len <= 0) {
        static const int bps = [] {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &nb, march3d_kernel<T, Ix, UNI, WRITE_RES, NW, MINB, PREF>, 32 * NW, 0) != cudaSuccess)
                nb = 0;
            return nb > 0 ? nb : 1;
        }();
        seg_len = m3_seg_len(tiles, e2 + 1, (long)num_sms * bps);
    }
    const int nseg = cg_div_up(e2 + 1, seg_len);
    return cg_launch(march3d_kernel<T, Ix, UNI, WRITE_RES, NW, MINB, PREF>, dim3((unsigned)(tiles * nseg)), dim3(32 * NW),
                     0, st, dep, f, s, e0, e1, e2, nstrip, nty, seg_len, s1u, s2u);
}

// Launch of the z-marching kernel over [0, n+1]^3; seg_len <= 0 picks the z-segment length;
// dep = true makes it a dependent launch (cg_launch).
// For FP32 with shared strides, variant 0 is 12 rows per block at 2 blocks per SM and variant 1
// is 8 rows per block at 3 blocks per SM (both 80 registers, no spills; the two best measured
// of 4-16 rows per block and 1-5 blocks per SM at 256^3).
template <class T, bool WRITE_RES>
inline cudaError_t launch_march3d(const Fused3D<T>& f, const SP<T>& s, int n0, int n1, int n2, int num_sms, int seg_len,
                                  cudaStream_t st, int variant = 0, bool dep = false) {
    long s1 = 0, s2 = 0;
    const bool uni = march3_uniform(f, &s1, &s2);
    if (march3_fits_int(f, n0 + 1, n1 + 1, n2 + 1)) {
        if (uni) {
            if constexpr (sizeof(T) == 4) {
                if (variant == 1)
                    return launch_march3d_ix<T, int, true, WRITE_RES, 3, 8>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, dep);
                return launch_march3d_ix<T, int, true, WRITE_RES, 2, 12>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, dep);
            }
            return launch_march3d_ix<T, int, true, WRITE_RES, 1>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, dep);
        }
        return launch_march3d_ix<T, int, false, WRITE_RES, 1>(f, s, n0, n1, n2, num_sms, seg_len, 0, 0, st, dep);
    }
    if (uni) return launch_march3d_ix<T, long, true, WRITE_RES, 1>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, dep);
    return launch_march3d_ix<T, long, false, WRITE_RES, 1>(f, s, n0, n1, n2, num_sms, seg_len, 0, 0, st, dep);
}

// ---- autotuner: the segment length (2D) or segment length and block shape (3D) with the
// shortest launch, timed with CUDA events on the caller's own buffers before a graph is
// captured. Only the `out` buffers of the ping-pong view are written (the first real iteration
// writes them again); the residual outputs are not touched. Results are cached per shape,
// precision and layout for the process.
// 2D candidates: variant 0 is march2d_kernel (one iteration per launch), variants 1 and 2 the
// two-iteration march2d_x2_kernel at 4 and 5 blocks per SM (when march_x2_ok); the time
// compared is per iteration.
template <class T>
inline cg_tune_cfg tune_march2d(const Fused2D<T>& f, const SP<T>& s, int n0, int n1, int nsm, cudaStream_t st) {
    cg_tune_cfg best{0, 0};
    if (cg_tune_forced(&best)) {
        if (best.variant > 2 || (best.variant >= 1 && !march_x2_ok(f, n0, n1))) best.variant = 0;
        return best;
    }
    if (!cg_autotune_enabled()) return best;
    std::string key = "march2d";
    cg_key_add(key, n0);
    cg_key_add(key, n1);
    cg_key_add(key, (int)sizeof(T));
    cg_key_add(key, march_uniform_stride(f));
    cg_key_add(key, nsm);
    cg_key_add(key, (int)march_x2_ok(f, n0, n1));
    if (cg_tune_lookup(key, &best)) return best;
    float tbest = 1e30f;
    for (int seg : {0, 8, 16, 24, 32, 48, 64}) {
        if (seg > n1 + 2) continue;
        const float t = time_launches([&] { return launch_march2d<T, false>(f, s, n0, n1, nsm, seg, st); }, st);
        if (cg_tune_verbose())
            std::fprintf(stderr, "march2d tune %dx%d: seg %d: %.1f us\n", n0, n1, seg, t >= 0.f ? 1e3f * t / 3 : -1.f);
        if (t >= 0.f && t < tbest) {
            tbest = t;
            best = cg_tune_cfg{seg, 0};
        }
    }
    if (march_x2_ok(f, n0, n1))
        for (int v : {1, 2})
            for (int seg : {0, 16, 32, 48, 64, 96}) {
                if (seg > n1 + 2) continue;
                float t = time_launches(
                    [&] { return launch_march2d_x2<T, false>(f, s, n0, n1, nsm, seg, true, st, false, v); }, st);
                if (t >= 0.f) t *= 0.5f;  // per iteration
                if (cg_tune_verbose())
                    std::fprintf(stderr, "march2d tune %dx%d: two iterations per pass (variant %d), seg %d: %.1f us per iteration\n",
                                 n0, n1, v, seg, t >= 0.f ? 1e3f * t / 3 : -1.f);
                if (t >= 0.f && t < tbest) {
                    tbest = t;
                    best = cg_tune_cfg{seg, v};
                }
            }
    cudaGetLastError();
    cg_tune_store(key, best);
    return best;
}

}  // namespace cgk
