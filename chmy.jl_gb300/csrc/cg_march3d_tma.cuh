// cg_march3d_tma.cuh — the fused 3D VE Stokes PT iteration (march3d_kernel's arithmetic,
// examples/stokes_3d_inc_ve_T.jl:23-57) with its input planes staged by the tensor memory
// accelerator.
//
// march3d_kernel issues one global load per input array per z-step, each with its own address
// and guard, and exchanges the old values its y-neighbours need through shared memory behind a
// block barrier. Here a producing warp of the block streams whole z-planes of the block's tile —
// every input array over the rows that read it — into a ring of S planes in shared memory with
// cp.async.bulk.tensor. The compute warps read their values and their y-neighbours' old values
// straight from the ring, so one barrier per plane remains among them (the exchange of the new
// values, double-buffered). Each ring slot has a `full` mbarrier (the copies' bytes arrive) and
// an `empty` mbarrier (every compute warp has read the plane); the producing warp refills a
// slot as soon as its `empty` phase completes, so no compute warp waits to issue copies.
//
// Parity: the warps compute exactly what march3d_kernel computes. Its loads read 0 where a guard
// is false; those guards bound x, y and z from above, and here every array's tensor map ends
// exactly where its guard ends, so the copies' zero fill gives the same 0. Values that only a
// halo row's unused results read (march3d_kernel's M3Need) are read from the ring as they fall.
//
// Failure handling: every wait is bounded by %globaltimer. A wait that runs out makes the compute
// warps stop at their next barrier (a barrier with a reduction, so all of them agree) and raise
// the error flag; the producing warp's wait for a release then runs out too, and it waits, again
// bounded, for its copies still in flight before it exits.
//
// Layout requirements (checked on the host): FP32, halo 1, every array with the same row and
// plane strides (multiples of 16 bytes) and the same offset from a 16-byte boundary.
#pragma once

#include "cg_march3d.cuh"
#include "cg_tma.cuh"

namespace m3t {

using namespace cgtma;

constexpr int kW = 36;  // box width: the warp's 32 columns from the 16-byte boundary at or before them
constexpr int kArrays = 21;
// Box order. The tensor components are (xx, yy, zz, xy, xz, yz); O* are the old stresses.
enum { VX, VY, VZ, IE, P, TYY, OYY, FP, TXX, TZZ, OXX, OZZ, TXY, OXY, TXZ, OXZ, TYZ, OYZ, RX, RY, RZ };

// First block row (warp) of array a's box and its number of rows for blocks of nw rows: the rows
// that read it (march3d_kernel's M3Need): V and 1/eta every row (the y-neighbours' old values
// included); P, tau_yy and the continuity forcing every row but the upper halo; tau_xy and tau_yz
// every row but the lower halo; the other diagonals, tau_xz and rho g the owned rows.
__host__ __device__ constexpr int row0(int a) { return a <= FP ? 0 : 1; }
__host__ __device__ constexpr int rows(int a, int nw) {
    return a <= IE    ? nw
           : a <= FP  ? nw - 1
           : a <= OZZ ? nw - 2
           : a <= OXY ? nw - 1
           : a <= OXZ ? nw - 2
           : a <= OYZ ? nw - 1
                      : nw - 2;
}
// Floats of array a's box in a ring slot (a multiple of 128 bytes) and its offset in the slot.
__host__ __device__ constexpr int box_floats(int a, int nw) { return (rows(a, nw) * kW + 31) / 32 * 32; }
__host__ __device__ constexpr int box_off(int a, int nw) {
    int o = 0;
    for (int b = 0; b < a; ++b) o += box_floats(b, nw);
    return o;
}
__host__ __device__ constexpr int slot_floats(int nw) { return box_off(kArrays, nw); }
// The arrays a segment reads at its first plane (ks - 1: the new P and tau_zz below plane ks,
// 1/eta below it) and at its last (ke + 1: V, 1/eta and the xz, yz shear inputs above plane ke);
// every other plane is read whole.
constexpr unsigned kFirstPlane = (1u << VX) | (1u << VY) | (1u << VZ) | (1u << IE) | (1u << P) | (1u << TZZ) |
                                 (1u << OZZ) | (1u << FP);
constexpr unsigned kLastPlane = (1u << VX) | (1u << VY) | (1u << VZ) | (1u << IE) | (1u << TXZ) | (1u << OXZ) |
                                (1u << TYZ) | (1u << OYZ);
// Bytes the copies of the arrays in `mask` deliver into one slot.
__host__ __device__ constexpr unsigned mask_bytes(unsigned mask, int nw) {
    unsigned b = 0;
    for (int a = 0; a < kArrays; ++a)
        if ((mask >> a) & 1u) b += (unsigned)(kW * rows(a, nw) * 4);
    return b;
}
// Dynamic shared memory of a block: 128 bytes to align the ring, S slots, two exchange buffers
// (P, tau_yy, tau_xy, tau_yz of every row) and 2 x S mbarriers.
__host__ __device__ constexpr int smem_bytes(int nw, int S) {
    return 128 + S * slot_floats(nw) * 4 + 2 * 4 * nw * 32 * 4 + 2 * S * 8;
}

struct Maps {
    CUtensorMap m[kArrays];
};

// The maps of one launch direction for blocks of nw rows.
struct Dir {
    bool ok = false;
    Maps maps;
    int xo = 0;             // tensor x of a field's first padded element
    unsigned tx = 0;        // bytes one ring slot's copies deliver
    unsigned present = 0;   // bit a: array a has a map (the forcing and rho g are optional)
};

}  // namespace m3t

namespace cgk {

// Barrier 1 over the first n threads of the block (the compute warps), returning whether any of
// them passed p = true; it orders their shared-memory accesses like __syncthreads.
__device__ __forceinline__ bool bar_or_compute(int n, bool p) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\tsetp.ne.u32 pi, %1, 0;\n\tbar.red.or.pred po, 1, %2, pi;\n\tselp.u32 %0, 1, 0, po;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(n)
        : "memory");
    return r != 0;
}

// The TMA-fed fused iteration. Block = NW compute warps over a tile of 30 x (NW - 2) owned
// (i, j) columns and one z segment, with march3d_kernel's lane and row assignment (lanes 0 and
// 31, warps 0 and NW-1 are one-point halos), and one producing warp (warp NW). Ring plane m is
// logical plane ks - 1 + m (tensor z = ks + m); array a's box in a slot starts at tensor
// (x0, j0 + row0(a)), x0 the 16-byte boundary at or before the tile's first column.
template <int NW, int MINB, int S, bool WRITE_RES>
__global__ void __launch_bounds__(32 * (NW + 1), MINB)
    march3d_tma_kernel(const __grid_constant__ m3t::Maps maps, const Fused3D<float> f, const SP<float> s, int e0, int e1,
                       int e2, int nstrip, int ntile_y, int seg_len, int s1u, int s2u, int xo, unsigned tx,
                       unsigned present, unsigned long long limit_ns, int withhold, int* err) {
    using namespace m3t;
    using T = float;
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int SF = slot_floats(NW);
    constexpr int XB = 4 * NW * 32;
    static_assert(S >= 3, "the ring holds the two planes a step reads and one in flight");
    extern __shared__ __align__(128) unsigned char smdyn[];
    unsigned char* smraw = smdyn + ((128u - (smem_u32(smdyn) & 127u)) & 127u);
    T* ring = reinterpret_cast<T*>(smraw);
    T* xb = ring + S * SF;
    uint64_t* full = reinterpret_cast<uint64_t*>(xb + 2 * XB);
    uint64_t* empty = full + S;
    cg_dep_wait();
    cg_dep_release();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int strip = b % nstrip, ty = (b / nstrip) % ntile_y, seg = b / (nstrip * ntile_y);
    const int ks = seg * seg_len;
    if (ks > e2) return;  // whole block, before any barrier exists
    const int ke = min(ks + seg_len - 1, e2);
    const int i0 = strip * 30, j0 = ty * (NW - 2);
    const int i = i0 - 1 + lane, j = j0 - 1 + w;
    const bool lo = w == 0, hi = w == NW - 1;
    const bool own = !lo && !hi && lane >= 1 && lane <= 30 && i <= e0 && j <= e1;
    const bool oldcell_ij = i < 0 || j < 0;  // column or row -1 keeps its old cells
    const MAt3<T, int, true> at{i, j, s1u, s2u};
    const int wu = w + 1 < NW ? w + 1 : NW - 1, wd = w > 0 ? w - 1 : 0;  // in-bounds neighbours
    const int ll = lane > 0 ? lane - 1 : 0;
    const int xs = i0 + xo;  // tensor x of lane 0's column
    const int bx0 = xs & ~3, cb = xs & 3;
    // the lane's element in rows w, w+1, w-1 of a box that starts at row 0, as a float offset
    const int pc = w * kW + cb + lane, pu = wu * kW + cb + lane, pd = wd * kW + cb + lane, pdl = wd * kW + cb + ll;
    const int nplanes = ke - ks + 3;  // planes ks-1 .. ke+1
    if (threadIdx.x == 0) {
        for (int q = 0; q < S; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], NW);
        }
        mbar_fence_init();
    }
    __syncthreads();  // the only barrier the producing warp takes part in
    if (w == NW) {
        // the producing warp: plane m goes into slot m % S once every compute warp has read
        // plane m - S from it, so each copy starts as early as the ring allows
        if (lane == 0) {
            int last[S];  // the last plane actually issued into each slot
            for (int q = 0; q < S; ++q) last[q] = -1;
            bool pok = true;
            for (int m = 0; m < nplanes && pok; ++m) {
                const int q = m % S;
                if (m >= S && !mbar_wait(&empty[q], (unsigned)((m - S) / S) & 1u, limit_ns)) {
                    pok = false;  // the compute warps stopped (or ran out of time)
                    break;
                }
                if (m == withhold) continue;  // a test's withheld plane: its waits run out
                const unsigned mask =
                    present & (m == 0 ? kFirstPlane : (m == nplanes - 1 ? kLastPlane : 0xffffffffu));
                T* dst = ring + q * SF;
                mbar_expect_tx(&full[q], mask == present ? tx : mask_bytes(mask, NW));
#pragma unroll
                for (int a = 0; a < kArrays; ++a)
                    if ((mask >> a) & 1u)
                        tma_load_3d(dst + box_off(a, NW), &maps.m[a], bx0, j0 + row0(a), ks + m, &full[q]);
                last[q] = m;
            }
            if (!pok) atomicExch(err, 1);
            // the copies still in flight complete before the block's shared memory goes away
            // (bounded; a slot's earlier planes completed before its last was issued)
            for (int q = 0; q < S; ++q)
                if (last[q] >= 0) mbar_wait(&full[q], (unsigned)(last[q] / S) & 1u, limit_ns);
        }
        return;
    }
    // array A of a slot at offset p of a box starting at row 0 (compile-time box offset)
#define M3T_R(sl, A, p) ((sl)[box_off(A, NW) - row0(A) * kW + (p)])

    bool ok = mbar_wait(&full[0], 0, limit_ns) && mbar_wait(&full[1], 0, limit_ns);
    // every decision to stop is taken by the whole warp (the shuffles below need all 32 lanes)
    ok = __all_sync(FULL, ok);

    // ---- prologue: new P, tau_zz at plane ks-1; new tau_xz, tau_yz at plane ks ----
    T vx_c, vy_c, vz_c, ie_c, ie_p, ieL_c, ieD_c, ieDL_c, Pn_p, tzzn_p, txz_c, tyz_c;
    {
        const T* s0 = ring;       // plane ks-1
        const T* s1 = ring + SF;  // plane ks
        const T vxp = M3T_R(s0, VX, pc), vyp = M3T_R(s0, VY, pc), vzp = M3T_R(s0, VZ, pc);
        const T iep = M3T_R(s0, IE, pc);
        const T pp = M3T_R(s0, P, pc), tzp = M3T_R(s0, TZZ, pc), tzop = M3T_R(s0, OZZ, pc);
        const T fpp = f.has_fP ? M3T_R(s0, FP, pc) : T(0);
        vx_c = M3T_R(s1, VX, pc);
        vy_c = M3T_R(s1, VY, pc);
        vz_c = M3T_R(s1, VZ, pc);
        ie_c = M3T_R(s1, IE, pc);
        const T txz0 = M3T_R(s1, TXZ, pc), txzo0 = M3T_R(s1, OXZ, pc);
        const T tyz0 = M3T_R(s1, TYZ, pc), tyzo0 = M3T_R(s1, OYZ, pc);
        const T vyUp = M3T_R(s0, VY, pu);  // Vy(i, j+1, ks-1)
        const T iepD = M3T_R(s0, IE, pd);  // 1/eta(i, j-1, ks-1)
        const T vzD = M3T_R(s1, VZ, pd);   // Vz(i, j-1, ks)
        ieD_c = M3T_R(s1, IE, pd);         // 1/eta(i, j-1, ks)
        ieDL_c = M3T_R(s1, IE, pdl);       // 1/eta(i-1, j-1, ks)
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[0]);  // this warp's last read of plane ks-1
        const T vxpR = __shfl_down_sync(FULL, vxp, 1);
        const Cell3<T> cp = m3_cell(s, f.has_fP != 0, rsub(vxpR, vxp), rsub(vyUp, vyp), rsub(vz_c, vzp), iep, pp, T(0),
                                    T(0), T(0), T(0), tzp, tzop, fpp);
        const bool keep = ks - 1 < 0 || oldcell_ij;
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
        if (own && ok) {
            at.st(f.tau_out[4], ks, txz_c);
            at.st(f.tau_out[5], ks, tyz_c);
        }
        ie_p = iep;
    }

    int sc = 1, sn = 2 % S;  // ring slots of planes k and k+1
    unsigned phn = 0;        // parity of plane k+1's fill of its slot
    for (int t = 0; t <= ke - ks; ++t) {
        const int k = ks + t;
        if (ok && !mbar_wait(&full[sn], phn, limit_ns)) ok = false;
        ok = __all_sync(FULL, ok);
        const T* slc = ring + sc * SF;
        const T* sln = ring + sn * SF;
        // plane k+1: V, 1/eta and the xz, yz shear inputs
        const T nvx = M3T_R(sln, VX, pc), nvy = M3T_R(sln, VY, pc), nvz = M3T_R(sln, VZ, pc), nie = M3T_R(sln, IE, pc);
        const T ntxz = M3T_R(sln, TXZ, pc), ntxzo = M3T_R(sln, OXZ, pc);
        const T ntyz = M3T_R(sln, TYZ, pc), ntyzo = M3T_R(sln, OYZ, pc);
        // plane k: the cell and xy inputs
        const T cP = M3T_R(slc, P, pc), ctyy = M3T_R(slc, TYY, pc), ctyo = M3T_R(slc, OYY, pc);
        const T cfp = f.has_fP ? M3T_R(slc, FP, pc) : T(0);
        const T ctxx = M3T_R(slc, TXX, pc), ctzz = M3T_R(slc, TZZ, pc), ctxo = M3T_R(slc, OXX, pc), ctzo = M3T_R(slc, OZZ, pc);
        const T ctxy = M3T_R(slc, TXY, pc), ctxyo = M3T_R(slc, OXY, pc);
        T crx = T(0), cry = T(0), crz = T(0);
        if (own) {
            if (f.has_rho[0]) crx = M3T_R(slc, RX, pc);
            if (f.has_rho[1]) cry = M3T_R(slc, RY, pc);
            if (f.has_rho[2]) crz = M3T_R(slc, RZ, pc);
        }
        // the y-neighbours' old values
        const T vyU = M3T_R(slc, VY, pu);     // Vy(i, j+1, k)
        const T vxD = M3T_R(slc, VX, pd);     // Vx(i, j-1, k)
        const T vzDn = M3T_R(sln, VZ, pd);    // Vz(i, j-1, k+1)
        const T ieDn = M3T_R(sln, IE, pd);    // 1/eta(i, j-1, k+1)
        const T ieDLn = M3T_R(sln, IE, pdl);  // 1/eta(i-1, j-1, k+1)
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[sc]);  // this warp's last read of plane k
        // new cell (i, j, k)
        const T vxR = __shfl_down_sync(FULL, vx_c, 1);
        Cell3<T> c = m3_cell(s, f.has_fP != 0, rsub(vxR, vx_c), rsub(vyU, vy_c), rsub(nvz, vz_c), ie_c, cP, ctxx, ctxo,
                             ctyy, ctyo, ctzz, ctzo, cfp);
        if (oldcell_ij) {
            c.P = cP;
            c.txx = ctxx;
            c.tyy = ctyy;
            c.tzz = ctzz;
        }
        // new tau_xy at (i, j, k): a = x, b = y
        const T vyL = __shfl_up_sync(FULL, vy_c, 1);
        const T txyn = (i > e0 || j > e1)
                           ? ctxy
                           : m3_shear(s, m3_rate(vx_c, vxD, s.idx[1], vy_c, vyL, s.idx[0]), ieDL_c, ieD_c, ieL_c, ie_c,
                                      ctxy, ctxyo);
        // new tau_xz, tau_yz at (i, j, k+1)
        const T vzLn = __shfl_up_sync(FULL, nvz, 1);
        const T ieLn = __shfl_up_sync(FULL, nie, 1);
        const T txzn = (i > e0 || k + 1 > e2)
                           ? ntxz
                           : m3_shear(s, m3_rate(nvx, vx_c, s.idx[2], nvz, vzLn, s.idx[0]), ieL_c, ie_c, ieLn, nie,
                                      ntxz, ntxzo);
        const T tyzn = (j > e1 || k + 1 > e2)
                           ? ntyz
                           : m3_shear(s, m3_rate(nvy, vy_c, s.idx[2], nvz, vzDn, s.idx[1]), ieD_c, ie_c, ieDn, nie,
                                      ntyz, ntyzo);
        // new values for the y-neighbours (the buffer of step t's parity: a warp is at most one
        // step ahead of another, since every step ends at the barrier below)
        T* xbk = xb + (t & 1) * XB;
        xbk[w * 32 + lane] = c.P;
        xbk[(NW + w) * 32 + lane] = c.tyy;
        xbk[(2 * NW + w) * 32 + lane] = txyn;
        xbk[(3 * NW + w) * 32 + lane] = tyz_c;
        __syncwarp();
        if (bar_or_compute(32 * NW, !ok)) {
            ok = false;
            break;
        }
        const T PD = xbk[wd * 32 + lane];               // P(i, j-1, k)
        const T tyyD = xbk[(NW + wd) * 32 + lane];      // tau_yy(i, j-1, k)
        const T txyU = xbk[(2 * NW + wu) * 32 + lane];  // tau_xy(i, j+1, k)
        const T tyzU = xbk[(3 * NW + wu) * 32 + lane];  // tau_yz(i, j+1, k)
        // velocity (i, j, k), as march3d_kernel
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
            if (f.has_rho[0]) rx = rsub(rx, crx);
            if (f.has_rho[1]) ry = rsub(ry, cry);
            if (f.has_rho[2]) rz = rsub(rz, crz);
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
        vx_c = nvx;
        vy_c = nvy;
        vz_c = nvz;
        ie_p = ie_c;
        ie_c = nie;
        ieL_c = ieLn;
        ieD_c = ieDn;
        ieDL_c = ieDLn;
        Pn_p = c.P;
        tzzn_p = c.tzz;
        txz_c = txzn;
        tyz_c = tyzn;
        sc = sn;
        if (++sn == S) {
            sn = 0;
            phn ^= 1u;
        }
    }
#undef M3T_R
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
}

}  // namespace cgk

namespace m3t {

// Maps of one launch direction for blocks of nw rows over the launch range [0, e]^3. fs: the
// input fields in box order (nullptr where absent; only FP and RX..RZ may be). Each map ends
// where march3d_kernel's guard of that array ends: V, 1/eta and the xz, yz shear inputs at
// logical e+1 in every dimension; tau_xy at e+1 in x and y and e in z; the cell inputs, the old
// stresses and rho g at e. Returns ok = false when a field's layout rules out tensor maps.
inline Dir make_dir(const cg_field* const fs[kArrays], int nw, int e0, int e1, int e2) {
    Dir d;
    int xo = -1;
    long s1 = 0, s2 = 0;
    for (int a = 0; a < kArrays; ++a) {
        const cg_field* fa = fs[a];
        if (!fa || !fa->data) {
            if (a == FP || a >= RX) continue;
            return Dir{};
        }
        const int o = map_offset(*fa);
        if (o < 0 || (xo >= 0 && o != xo)) return Dir{};
        if (fa->halo[0] != 1 || fa->halo[1] != 1 || fa->halo[2] != 1) return Dir{};
        if (xo < 0) {
            s1 = fa->stride[1];
            s2 = fa->stride[2];
        } else if (fa->stride[1] != s1 || fa->stride[2] != s2) {
            return Dir{};
        }
        xo = o;
        const bool vx = a <= IE || a == TXZ || a == TYZ || a == TXY;  // readable to e+1 in x and y
        const bool vz = a <= IE || a == TXZ || a == TYZ;              // readable to e+1 in z
        // logical index L is tensor index L + 1 (+ xo along x)
        const cuuint64_t ext[3] = {(cuuint64_t)(e0 + (vx ? 3 : 2) + xo), (cuuint64_t)(e1 + (vx ? 3 : 2)),
                                   (cuuint64_t)(e2 + (vz ? 3 : 2))};
        if (!make_map_ext(*fa, xo, ext, kW, rows(a, nw), &d.maps.m[a])) return Dir{};
        d.present |= 1u << a;
        d.tx += (unsigned)(kW * rows(a, nw) * 4);
    }
    d.xo = xo;
    d.ok = true;
    return d;
}

// The input fields of a fused view's direction in box order.
inline void dir_fields(const cg_field* const V[3], const cg_field* ie, const cg_field* Pf, const cg_field* const tau[6],
                       const cg_field* const told[6], const cg_field* fP, const cg_field* const rho[3],
                       const cg_field* out[kArrays]) {
    out[VX] = V[0];
    out[VY] = V[1];
    out[VZ] = V[2];
    out[IE] = ie;
    out[P] = Pf;
    out[TYY] = tau[1];
    out[OYY] = told[1];
    out[FP] = fP;
    out[TXX] = tau[0];
    out[TZZ] = tau[2];
    out[OXX] = told[0];
    out[OZZ] = told[2];
    out[TXY] = tau[3];
    out[OXY] = told[3];
    out[TXZ] = tau[4];
    out[OXZ] = told[4];
    out[TYZ] = tau[5];
    out[OYZ] = told[5];
    out[RX] = rho[0];
    out[RY] = rho[1];
    out[RZ] = rho[2];
}

// Block heights of the TMA variants (march3d variants 2 and 3).
constexpr int kHeights = 2;
constexpr int kHeight[kHeights] = {12, 8};

// Maps for both ping-pong directions of a fused 3D loop and every TMA block height, and the
// device flag a kernel raises when a wait runs out.
struct Tma {
    bool ok = false;
    Dir ab[kHeights], ba[kHeights];
    int* err = nullptr;
};

// The maps of a ping-pong pair of field sets: direction ab reads (Va, Pa, taua), direction ba
// reads (Vb, Pb, taub); 1/eta, the old stresses, the forcing and rho g are shared (nullptr:
// absent). ok = false where a layout rules out tensor maps (the register-fed variants remain).
inline Tma make_tma(const cg_field* const Va[3], const cg_field* Pa, const cg_field* const taua[6],
                    const cg_field* const Vb[3], const cg_field* Pb, const cg_field* const taub[6], const cg_field* ie,
                    const cg_field* const told[6], const cg_field* fP, const cg_field* const rho[3], const int n[3],
                    int* err) {
    Tma t;
    t.err = err;
    t.ok = err != nullptr;
    const int e0 = n[0] + 1, e1 = n[1] + 1, e2 = n[2] + 1;
    const cg_field* fa[kArrays];
    const cg_field* fb[kArrays];
    dir_fields(Va, ie, Pa, taua, told, fP, rho, fa);
    dir_fields(Vb, ie, Pb, taub, told, fP, rho, fb);
    for (int h = 0; h < kHeights && t.ok; ++h) {
        t.ab[h] = make_dir(fa, kHeight[h], e0, e1, e2);
        t.ba[h] = make_dir(fb, kHeight[h], e0, e1, e2);
        t.ok = t.ab[h].ok && t.ba[h].ok;
    }
    return t;
}

}  // namespace m3t

namespace cgk {

// Which direction's maps a launch uses (nullptr: none, the register-fed variants only).
struct M3Launch {
    const m3t::Dir* dir[m3t::kHeights] = {nullptr, nullptr};
    int* err = nullptr;
};

inline M3Launch m3_launch_of(const m3t::Tma* t, bool ab) {
    M3Launch l;
    if (!t || !t->ok) return l;
    for (int h = 0; h < m3t::kHeights; ++h) l.dir[h] = ab ? &t->ab[h] : &t->ba[h];
    l.err = t->err;
    return l;
}

// The TMA-fed iteration with blocks of NW rows, a ring of S planes and at most MINB blocks per
// SM by its launch bounds.
template <int NW, int MINB, int S, bool WRITE_RES>
inline cudaError_t launch_march3d_tma(const Fused3D<float>& f, const SP<float>& s, int n0, int n1, int n2, int num_sms,
                                      int seg_len, long s1u, long s2u, cudaStream_t st, bool dep, const m3t::Dir& d,
                                      int* err) {
    auto kern = march3d_tma_kernel<NW, MINB, S, WRITE_RES>;
    constexpr int smem = m3t::smem_bytes(NW, S);
    static_assert(smem <= 232448, "the ring exceeds a block's shared memory");
    // set on every launch (launches happen while tuning and capturing graphs): each translation
    // unit that launches the kernel has its own copy of it, while a static in this inline
    // function would be shared by all of them
    cudaError_t ae = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (ae != cudaSuccess) return ae;
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 32 * (NW + 1), smem) != cudaSuccess || bps < 1) {
        cudaGetLastError();
        bps = 1;
    }
    const int e0 = n0 + 1, e1 = n1 + 1, e2 = n2 + 1;
    const int nstrip = cg_div_up(e0 + 1, 30), nty = cg_div_up(e1 + 1, NW - 2);
    const long tiles = (long)nstrip * nty;
    if (seg_len <= 0) seg_len = m3_seg_len(tiles, e2 + 1, (long)num_sms * bps);
    const int nseg = cg_div_up(e2 + 1, seg_len);
    const cg_tma_cfg wc = cg_tma_wait_cfg();
    return cg_launch(kern, dim3((unsigned)(tiles * nseg)), dim3(32 * (NW + 1)), (size_t)smem, st, dep, d.maps, f, s, e0, e1, e2,
                     nstrip, nty, seg_len, (int)s1u, (int)s2u, d.xo, d.tx, d.present, wc.limit_ns, wc.withhold, err);
}

// Variants of the fused 3D iteration: 0 and 1 march3d_kernel (12 rows at 2 blocks per SM, 8 rows
// at 3); 2 and 3 march3d_tma_kernel (12 rows at 2 blocks per SM, 8 rows at 3, rings of 3 planes),
// only with the direction's tensor maps and otherwise variant 0.
constexpr int kM3Variants = 4;
constexpr int kM3TmaFirst = 2;

template <class T, bool WRITE_RES>
inline cudaError_t launch_march3d_any(const Fused3D<T>& f, const SP<T>& s, int n0, int n1, int n2, int num_sms,
                                      int seg_len, cudaStream_t st, int variant, bool dep, const M3Launch& l) {
    if constexpr (sizeof(T) == 4) {
        if (variant >= kM3TmaFirst) {
            const int h = variant - kM3TmaFirst;
            long s1 = 0, s2 = 0;
            if (h < m3t::kHeights && l.dir[h] && l.dir[h]->ok && l.err && march3_uniform(f, &s1, &s2) &&
                march3_fits_int(f, n0 + 1, n1 + 1, n2 + 1)) {
                // an ordinary launch (and the bc! launch after it too): with dependent launches around
                // it, the defect-correction chunk measured 465-486 instead of 457-472 us per 256^3
                // iteration
                if (h == 0)
                    return launch_march3d_tma<12, 2, 3, WRITE_RES>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, false,
                                                                   *l.dir[0], l.err);
                return launch_march3d_tma<8, 3, 3, WRITE_RES>(f, s, n0, n1, n2, num_sms, seg_len, s1, s2, st, false,
                                                              *l.dir[1], l.err);
            }
            variant = 0;
        }
    }
    return launch_march3d<T, WRITE_RES>(f, s, n0, n1, n2, num_sms, seg_len, st, variant >= kM3TmaFirst ? 0 : variant, dep);
}

// The autotuner of the fused 3D iteration: segment length and variant (the TMA variants where
// the direction's maps exist), timed like tune_march2d.
template <class T>
inline cg_tune_cfg tune_march3d(const Fused3D<T>& f, const SP<T>& s, int n0, int n1, int n2, int nsm, cudaStream_t st,
                                const M3Launch& l = M3Launch{}) {
    cg_tune_cfg best{0, 0};
    const bool tma = sizeof(T) == 4 && l.dir[0] && l.dir[0]->ok && l.err;
    if (cg_tune_forced(&best)) {
        if (best.variant >= kM3TmaFirst && !tma) best.variant = 0;
        return best;
    }
    if (!cg_autotune_enabled()) return best;
    long s1 = 0, s2 = 0;
    const bool uni = march3_uniform(f, &s1, &s2);
    std::string key = "march3d";
    cg_key_add(key, n0);
    cg_key_add(key, n1);
    cg_key_add(key, n2);
    cg_key_add(key, (int)sizeof(T));
    cg_key_add(key, uni ? s1 : 0L);
    cg_key_add(key, uni ? s2 : 0L);
    cg_key_add(key, nsm);
    cg_key_add(key, (int)tma);
    if (cg_tune_lookup(key, &best)) return best;
    const int nvar = (sizeof(T) == 4 && uni) ? (tma ? kM3Variants : 2) : 1;
    float tbest = 1e30f;
    for (int v = 0; v < nvar; ++v)
        for (int seg : {0, 16, 32, 64}) {
            if (seg > n2 + 2) continue;
            const float t = time_launches(
                [&] { return launch_march3d_any<T, false>(f, s, n0, n1, n2, nsm, seg, st, v, false, l); }, st);
            if (cg_tune_verbose())
                std::fprintf(stderr, "march3d tune %dx%dx%d: seg %d variant %d: %.1f us\n", n0, n1, n2, seg, v,
                             t >= 0.f ? 1e3f * t / 3 : -1.f);
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
