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

using cgk::bits_of;

using cgk::block_max_bits;

}  // namespace cgsia
