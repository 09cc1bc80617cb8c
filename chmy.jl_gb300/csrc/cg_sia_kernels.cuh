// cg_sia_kernels.cuh — device arithmetic shared by the single-member and ensemble shallow-ice
// solvers (Chmy.jl examples/sia.jl:30-54).
//
// The SIA step runs in FP64, and on GB300 it is bound by the FP64 pipe, not by HBM: a cell
// needs tens of FP64 instructions for 24 bytes of traffic. The arithmetic is therefore
// arranged to issue as few FP64 instructions as possible.
// - Integer powers use repeated squaring.
// - For odd n, vmag(∇S)^(n-1) is an integer power of |∇S|^2, with no square root.
// - D = h^n (Gamma h^2 + As) |∇S|^(n-1) shares the h^n factor of the reference's
//   Gamma h^(n+2) + As h^n.
// These forms differ from the reference's evaluation order only in rounding, a few ulp.
// The maximum of D over a member, which sets the adaptive Δt, is reduced within a block first
// (warp shuffles, then shared memory). One atomic per block then updates the member's slot,
// where an atomic per cell would serialise on a single address.
#pragma once

#include "cg_common.cuh"

namespace cgsia {

// x^m for m >= 0 by repeated squaring (x^1 is x itself, with no multiplication)
template <class T>
__device__ __forceinline__ T pow_int(T x, int m) {
    T r = (m & 1) ? x : T(1);
    m >>= 1;
    while (m) {
        x = x * x;
        if (m & 1) r = r * x;
        m >>= 1;
    }
    return r;
}

// D = (Gamma h^(n+2) + As h^n) vmag^(n-1) at a cell, where vmag^2 = ax^2 + ay^2 and ax, ay are
// the components of ∇S interpolated to the cell (examples/sia.jl:46-49).
template <class T>
__device__ __forceinline__ T D_cell(T h, T ax, T ay, T Gamma, T As, int n) {
    const T vm2 = ax * ax + ay * ay;
    const int e = n - 1;
    T vp = pow_int(vm2, e >> 1);
    if (e & 1) vp = vp * sqrt(vm2);
    return pow_int(h, n) * fma(Gamma, h * h, As) * vp;
}

// D at a cell (bit for bit the value of D_cell) and the derivatives a taped forward step
// records, from the same subexpressions: dD/dh, c ax and c ay with c = 2 dD/dV (V = ax^2 + ay^2;
// these are dD/dax and dD/day), and dD/dGamma = h^(n+2) V^((n-1)/2). Gn2 = Gamma (n+2) and
// Asn = As n are the caller's constants.
template <class T>
__device__ __forceinline__ T D_and_factors(T h, T ax, T ay, T Gamma, T As, T Gn2, T Asn, int n, T* dh, T* ex, T* ey,
                                           T* gf) {
    const T V = ax * ax + ay * ay;
    const int e = n - 1;
    T vp = pow_int(V, e >> 1);
    if (e & 1) vp = vp * sqrt(V);
    const T h2 = h * h;
    const T hn = pow_int(h, n);
    const T A = hn * fma(Gamma, h2, As);
    const T D = A * vp;
    T c = T(0);
    if (n >= 3) {
        T vq = pow_int(V, (n - 3) >> 1);
        if ((n - 3) & 1) vq = vq * sqrt(V);
        c = A * T(n - 1) * vq;
    } else if (n == 2 && V > T(0)) {
        c = A / sqrt(V);
    }
    *dh = fma(Gn2, h2, Asn) * pow_int(h, n - 1) * vp;
    *ex = c * ax;
    *ey = c * ay;
    *gf = hn * h2 * vp;
    return D;
}

using cgk::bits_of;

using cgk::block_max_bits;

// Sum over the block (valid in thread 0). Every thread calls it; it may be called more than
// once per kernel (the leading barrier keeps a call's writes after the previous call's reads).
__device__ __forceinline__ double block_sum(double x) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ double part[32];
    __syncthreads();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5, nw = (blockDim.x * blockDim.y + 31) >> 5;
    if (lane == 0) part[warp] = x;
    __syncthreads();
    x = 0.0;
    if (warp == 0) {
        x = lane < nw ? part[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    }
    return x;  // valid in thread 0
}

// ---- tape of a forward run, read by the reverse sweep ---------------------------------------
//
// A taped forward step records what the reverse step would otherwise recompute in FP64. This
// trades HBM traffic, which the SIA kernels barely use, for FP64 instructions, which bound them.
// Layout: a 256-byte header, then per step a 256-byte word block and kArrays arrays of `cnt`
// elements in H's padded layout (each rounded up to 256 bytes).
enum TapeArray {
    kD = 0,   // D over cells [0, n]^2
    kGX = 1,  // dS/dx at the cell's lower x face ((S_i - S_i-1)/dx)
    kGY = 2,  // dS/dy at the lower y face
    kDH = 3,  // dD/dh
    kEX = 4,  // dD/dax = 2 dD/dV ax  (V = ax^2 + ay^2)
    kEY = 5,  // dD/day = 2 dD/dV ay
    kGF = 6,  // dD/dGamma = h^(n+2) V^((n-1)/2)
    kW = 7,   // W = -divg(q) + M
    kFL = 8,  // one byte per cell: 1 if H + dt W > 0, plus 2 if the mass balance is not capped
    kArrays = 9
};

struct TapeHeader {
    unsigned long long magic;
    int dtype, nx, ny, nsteps;
    long long stride0, stride1, halo0, halo1, n0, n1, cnt, step_bytes;
    double Gamma, As, beta, ela, m_max, cfl, dt_max;
    int n, pad;
};
constexpr unsigned long long kTapeMagic = 0x3145504154414953ull;  // "SIATAPE1"

// per step: the forward's Dmax bits, the first interior argmax (j (nx+2) + i), dt and whether
// dt was capped at dt_max
struct TapeWords {
    unsigned long long dmax;
    unsigned long long arg;
    double dt;
    double capped;
};

struct TapeGeom {
    size_t cnt, abytes, step_bytes;
};

// elements per array: H's allocation (row stride x padded rows)
inline TapeGeom tape_geom(const cg_field& H, size_t elem) {
    TapeGeom g;
    g.cnt = (size_t)H.stride[1] * (size_t)(H.n[1] + 4 * H.halo[1]);
    g.abytes = (g.cnt * elem + 255) & ~(size_t)255;
    g.step_bytes = 256 + (size_t)kArrays * g.abytes;
    return g;
}

}  // namespace cgsia
