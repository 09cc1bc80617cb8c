// cg_stokes_adjoint.cu — gradient of a velocity misfit with respect to log-viscosity for the
// steady VE Stokes step (examples/stokes_{2,3}d_inc_ve_T.jl, variable-viscosity form).
//
// With tau eliminated, one PT step solves K (V, P) = b, where
//   K = [[L, -G], [-G^T, 0]],  L V = div(2 eta_ve dev(eps(V))) = -E^T W (2 eta_ve Pdev) E V,
// E is the staggered strain-rate operator, G the pressure gradient, W weighs shear components
// twice (each appears in two momentum equations) and Pdev takes the deviator of the diagonal
// components. On the staggered grid div and grad are negative transposes of each other, so K is
// symmetric. For a misfit J(V) the adjoint mu therefore solves the same Stokes problem,
// K mu = -dJ/dV: the forward PT solver with body force -dJ/dV, tau_old = 0 and the forward's
// boundary-condition kinds with zero values. With m = log(eta), 1/eta = exp(-m) and
// eta_ve = 1/(1/eta + 1/(G dt)):
//   dJ/dm = mu^T dK/dm (V, P) - mu^T db/dm
//         = -sum over stress locations of w (d eta_ve/dm) / eta_ve * eps(mu) . tau(V),
// with tau(V) = eta_ve (2 dev(eps(V)) + tau_old/(G dt)), the constitutive stress of the converged
// velocity. It is evaluated from V itself: the reference's convergence test bounds only the
// momentum and continuity residuals, so the PT stress can still carry a divergence-free error
// that leaves V unchanged. At a cell (d eta_ve/dm_c)/eta_ve = eta_ve (1/eta)_c; at a shear edge,
// whose 1/eta is the mean of its 4 cells, it is eta_ve_e (1/eta)_c / 4 for each of them. Hence,
// per interior cell c,
//   dJ/dm_c = -(1/eta)_c [ eta_ve_c sum_d eps_dd(mu) tau_dd(V) + 1/2 sum_{edges e at c}
//                          eta_ve_e eps_e(mu) tau_e(V) ].
// The interior cells are the logical indices 1..n, and the shear edges at a cell are its lower
// and upper vertex of each pair of dimensions, all within the edges' interior 1..n+1. This file
// computes that sum; the adjoint solve is an ordinary cg_stokes_solve.
#include "cg_common.cuh"
#include "cg_stokes_kernels.cuh"

namespace {
using namespace cgk;

template <class T>
struct GradArgs {
    DF<T> mu[3];      // adjoint velocity
    DF<T> V[3];       // converged forward velocity
    DF<T> tau_o[6];   // forward tau_old (has_told)
    DF<T> eta, ieta;  // viscosity or its inverse (has_ieta picks)
    DF<T> grad;       // dJ/d log(eta) at cells
    T inv_Gdt, idx[3];
    int has_ieta, has_told;
    __device__ __forceinline__ T inv_eta(int i, int j, int k) const {
        return has_ieta ? ieta(i, j, k) : T(1) / eta(i, j, k);
    }
};

// 1/eta on the (a, b) edge at point (i, j, k): the Linear rule over its 4 cells.
template <class T>
__device__ __forceinline__ T edge_ieta(const GradArgs<T>& g, int i, int j, int k, int a, int b) {
    const int ai = a == 0, aj = a == 1, ak = a == 2;
    const int bi = b == 0, bj = b == 1, bk = b == 2;
    const T e00 = g.inv_eta(i - ai - bi, j - aj - bj, k - ak - bk);
    const T e10 = g.inv_eta(i - bi, j - bj, k - bk);
    const T e01 = g.inv_eta(i - ai, j - aj, k - ak);
    const T e11 = g.inv_eta(i, j, k);
    const T lo = fma(T(0.5), e10 - e00, e00);
    const T hi = fma(T(0.5), e11 - e01, e01);
    return fma(T(0.5), hi - lo, lo);
}

// Shear strain rate 0.5 (d_b(U_a) + d_a(U_b)) of the velocity U on the (a, b) edge at I: U_a is
// Center along b, so d_b(U_a) = U_a[I] - U_a[I - e_b]; likewise d_a(U_b).
template <class T>
__device__ __forceinline__ T edge_rate(const DF<T>* U, const T* idx, int i, int j, int k, int a, int b) {
    int Ib[3] = {i, j, k}, Ia[3] = {i, j, k};
    Ib[b] -= 1;
    Ia[a] -= 1;
    const T dba = (U[a](i, j, k) - U[a](Ib[0], Ib[1], Ib[2])) * idx[b];
    const T dab = (U[b](i, j, k) - U[b](Ia[0], Ia[1], Ia[2])) * idx[a];
    return T(0.5) * (dba + dab);
}

// eta_ve * eps_ab(mu) * tau_ab(V) on the (a, b) edge at point (i, j, k), tau component c.
template <class T>
__device__ __forceinline__ T edge_term(const GradArgs<T>& g, int i, int j, int k, int a, int b, int c) {
    const T eve = T(1) / (edge_ieta(g, i, j, k, a, b) + g.inv_Gdt);
    T src = T(2) * edge_rate(g.V, g.idx, i, j, k, a, b);
    if (g.has_told) src += g.tau_o[c](i, j, k) * g.inv_Gdt;
    return eve * edge_rate(g.mu, g.idx, i, j, k, a, b) * (eve * src);
}

// One thread per interior cell: logical indices 1..n (0 and n+1 are the ghost layers of the
// launch range [0, n+1]).
template <class T, int ND>
__global__ void grad_log_eta_kernel(const GradArgs<T> g, int n0, int n1, int n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = ND > 2 ? blockIdx.z + 1 : 0;
    if (i > n0 || j > n1 || (ND > 2 && k > n2)) return;
    const T ie = g.inv_eta(i, j, k);
    const T eve = T(1) / (ie + g.inv_Gdt);
    // diagonal: eps_dd(mu) tau_dd(V) at the cell, tau_dd(V) = eta_ve (2 (eps_dd - div/3) + tau_old/(G dt))
    T em[3], ev[3], dv = T(0);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        int I1[3] = {i, j, k};
        I1[d] += 1;
        em[d] = (g.mu[d](I1[0], I1[1], I1[2]) - g.mu[d](i, j, k)) * g.idx[d];
        ev[d] = (g.V[d](I1[0], I1[1], I1[2]) - g.V[d](i, j, k)) * g.idx[d];
        dv += ev[d];
    }
    T sd = T(0);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        T src = T(2) * (ev[d] - dv / T(3));
        if (g.has_told) src += g.tau_o[d](i, j, k) * g.inv_Gdt;
        sd += em[d] * (eve * src);
    }
    // shear: the 4 edges of each (a, b) component around the cell
    T ss = T(0);
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int q = 0; q < (ND == 2 ? 1 : 3); ++q) {
        const int a = pairs[q][0], b = pairs[q][1];
        const int c = ND == 2 ? 2 : 3 + q;
        for (int s = 0; s < 4; ++s) {
            int E[3] = {i, j, k};
            E[a] += s & 1;
            E[b] += (s >> 1) & 1;
            ss += edge_term(g, E[0], E[1], E[2], a, b, c);
        }
    }
    g.grad(i, j, k) = -ie * (eve * sd + T(0.5) * ss);
}

template <class T, int ND>
int launch_grad(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* fwd, const cg_field* mu,
                const cg_stokes_params* p, const cg_field* grad) {
    GradArgs<T> g;
    std::memset(&g, 0, sizeof(g));
    for (int d = 0; d < ND; ++d) {
        g.mu[d] = cg_view<T>(mu[d]);
        g.idx[d] = (T)grid->inv_spacing[d];
    }
    for (int d = 0; d < ND; ++d) g.V[d] = cg_view<T>(fwd->V[d]);
    g.has_told = cg_present(fwd->tau_old[0]);
    if (g.has_told)
        for (int c = 0; c < (ND == 2 ? 3 : 6); ++c) g.tau_o[c] = cg_view<T>(fwd->tau_old[c]);
    if (cg_present(fwd->inv_eta)) {
        g.ieta = cg_view<T>(fwd->inv_eta);
        g.has_ieta = 1;
    } else {
        g.eta = cg_view<T>(fwd->eta);
    }
    g.grad = cg_view<T>(*grad);
    g.inv_Gdt = T(1) / ((T)p->G * (T)p->dt);
    dim3 block(32, 8);
    dim3 gr(cg_div_up(grid->n[0], block.x), cg_div_up(grid->n[1], block.y), ND > 2 ? grid->n[2] : 1);
    grad_log_eta_kernel<T, ND><<<gr, block, 0, ctx->stream>>>(g, grid->n[0], grid->n[1], ND > 2 ? grid->n[2] : 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

}  // namespace

extern "C" int cg_stokes_gradient_log_eta(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* fwd,
                                          const cg_field* mu, const cg_stokes_params* p, const cg_field* grad) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "stokes_gradient_log_eta: ctx is NULL");
    if (!grid || !fwd || !mu || !p || !grad) return cg_fail(ctx, CG_ERR_ARG, "stokes_gradient_log_eta: NULL argument");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    const int nd = grid->ndim;
    if (nd < 2) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_gradient_log_eta: 2D and 3D grids only");
    const int dtype = grad->dtype;
    if ((rc = cg_check_field(ctx, grid, *grad, dtype, 0, "grad"))) return rc;
    if (cg_present(fwd->inv_eta)) {
        if ((rc = cg_check_field(ctx, grid, fwd->inv_eta, dtype, 0, "inv_eta"))) return rc;
    } else if (cg_present(fwd->eta)) {
        if ((rc = cg_check_field(ctx, grid, fwd->eta, dtype, 0, "eta"))) return rc;
    } else {
        return cg_fail(ctx, CG_ERR_ARG, "stokes_gradient_log_eta: a viscosity field (eta or inv_eta) is required");
    }
    for (int d = 0; d < nd; ++d)
        if ((rc = cg_check_field(ctx, grid, mu[d], dtype, 1 << d, "mu (adjoint velocity)"))) return rc;
    for (int d = 0; d < nd; ++d)
        if ((rc = cg_check_field(ctx, grid, fwd->V[d], dtype, 1 << d, "V"))) return rc;
    const int nt = nd == 2 ? 3 : 6;
    const int shear2[3] = {0, 0, 0b11}, shear3[6] = {0, 0, 0, 0b011, 0b101, 0b110};
    if (cg_present(fwd->tau_old[0]))
        for (int c = 0; c < nt; ++c)
            if ((rc = cg_check_field(ctx, grid, fwd->tau_old[c], dtype, nd == 2 ? shear2[c] : shear3[c], "tau_old")))
                return rc;
    cudaSetDevice(ctx->device);
    if (dtype == CG_F64)
        return nd == 2 ? launch_grad<double, 2>(ctx, grid, fwd, mu, p, grad)
                       : launch_grad<double, 3>(ctx, grid, fwd, mu, p, grad);
    return nd == 2 ? launch_grad<float, 2>(ctx, grid, fwd, mu, p, grad) : launch_grad<float, 3>(ctx, grid, fwd, mu, p, grad);
}
