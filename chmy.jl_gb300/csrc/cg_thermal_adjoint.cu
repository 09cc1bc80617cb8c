// cg_thermal_adjoint.cu — vector-Jacobian product of the fused thermal step
// (update_thermal_flux! + update_thermal!, examples/stokes_2d_inc_ve_T.jl:45-60, then bc!(T)).
//
// Forward, at an interior cell c (every face flux it reads lies in the flux kernel's range):
//   T_out[c] = T_old[c] - dt sum_d (q_d[c + e_d] - q_d[c]) idx_d
//   q_d[J] = -lambda (T[J] - T[J - e_d]) idx_d + max(V_d[J], 0) T[J - e_d] + min(V_d[J], 0) T[J]
// For a misfit J of T_out's interior cells with mu = dJ/dT_out there (zero elsewhere), a face J
// between cells l = J - e_d and r = J carries nu_d[J] = dJ/dq_d[J] = dt idx_d (mu[r] - mu[l]),
// and
//   dJ/dT[l] += nu (lambda idx + max'(V) ... ), dJ/dT[r] += nu (-lambda idx + min'(V) ...)
//   dJ/dV_d[J] = nu (T[l] [V >= 0] + T[r] [V <= 0])         (the kernel's branches at V = 0)
//   dJ/dlambda += nu (-(T[r] - T[l]) idx)
//   dJ/dT_old[c] = mu[c].
// The ghost cells of T are the bc_T rules' functions of the interior (T came from a step that
// ended with bc!(T)): a ghost's term is folded into the cell it follows (Neumann +1, Dirichlet
// on a Center field -1, Periodic: the opposite cell). Each thread owns one interior cell: its
// left faces (and its right faces on the last cell of a dimension), so no two threads write one
// address; dJ/dlambda is summed in FP64 per block in a fixed order (warp shuffles, then the
// warps in order) and, when the caller asks for it, over the blocks in a fixed order.
#include "cg_common.cuh"

namespace {

constexpr int kThermalSlot = 9;  // ctx scratch slot: per-block dJ/dlambda partials and their sum

template <class T>
struct ThermalAdj {
    DF<T> Tin, mu, gT, gTold, gV[3];
    DF<T> V[3];
    double* gacc;
    T lam, dt, idx[3];
    int rule[3][2];  // +1 Neumann, -1 Dirichlet, 2 Periodic
    int n[3];
    int has_gTold;
};

template <class T>
__device__ __forceinline__ T vpos(T v) {  // d max(v, 0)/dv as the kernel's branch takes it
    return v < T(0) ? T(0) : T(1);
}
template <class T>
__device__ __forceinline__ T vneg1(T v) {  // d min(v, 0)/dv
    return T(0) < v ? T(0) : T(1);
}

// Sum of a block's per-thread values in a fixed order (warp shuffles, then the warps in order),
// written to part[block]: the same bits on every run.
__device__ __forceinline__ void block_sum_fixed(double v, double* part) {
    __shared__ double warp_part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((t & 31) == 0) warp_part[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += warp_part[w];
        part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// The cell (i, j, k)'s outputs; returns its dJ/dlambda term.
template <class T, int ND>
__device__ __forceinline__ double thermal_adjoint_cell(const ThermalAdj<T>& a, int i, int j, int k) {
    const int c[3] = {i, j, k};
    const T mc = a.mu(i, j, k);
    const T tc = a.Tin(i, j, k);
    T g = T(0);
    double dl = 0.0;
    for (int d = 0; d < ND; ++d) {
        int L[3] = {i, j, k}, R[3] = {i, j, k};
        L[d] -= 1;
        R[d] += 1;
        const bool first = c[d] == 1, last = c[d] == a.n[d];
        const T ml = first ? T(0) : a.mu(L[0], L[1], L[2]);
        const T mr = last ? T(0) : a.mu(R[0], R[1], R[2]);
        const T s = a.dt * a.idx[d];
        const T nuL = s * (mc - ml), nuR = s * (mr - mc);
        const T vL = a.V[d](i, j, k), vR = a.V[d](R[0], R[1], R[2]);
        const T li = a.lam * a.idx[d];
        // c is the right cell of its left face and the left cell of its right face
        g += nuR * (li + (vR < T(0) ? T(0) : vR)) + nuL * (-li + (T(0) < vL ? T(0) : vL));
        // the ghost beside c along d (Neumann / Dirichlet): its one face is c's boundary face
        if (first && a.rule[d][0] != 2) g += T(a.rule[d][0]) * nuL * (li + (vL < T(0) ? T(0) : vL));
        if (last && a.rule[d][1] != 2) g += T(a.rule[d][1]) * nuR * (-li + (T(0) < vR ? T(0) : vR));
        // Periodic: the ghost left of the first cell is this dimension's last cell, and the
        // ghost right of the last cell is its first cell
        if (last && a.rule[d][0] == 2) {
            int F[3] = {i, j, k};
            F[d] = 1;
            const T mf = a.mu(F[0], F[1], F[2]);
            const T vf = a.V[d](F[0], F[1], F[2]);
            g += (s * mf) * (li + (vf < T(0) ? T(0) : vf));
        }
        if (first && a.rule[d][1] == 2) {
            int Ls[3] = {i, j, k}, Rn[3] = {i, j, k};
            Ls[d] = a.n[d];
            Rn[d] = a.n[d] + 1;
            const T mlast = a.mu(Ls[0], Ls[1], Ls[2]);
            const T vlast = a.V[d](Rn[0], Rn[1], Rn[2]);
            g += (-s * mlast) * (-li + (T(0) < vlast ? T(0) : vlast));
        }
        // faces owned by c: its left face, and its right face on the last cell
        const T tl = a.Tin(L[0], L[1], L[2]);
        a.gV[d](i, j, k) = nuL * (tl * vpos(vL) + tc * vneg1(vL));
        dl += (double)nuL * (-(double)(tc - tl) * (double)a.idx[d]);
        if (last) {
            const T tr = a.Tin(R[0], R[1], R[2]);
            a.gV[d](R[0], R[1], R[2]) = nuR * (tc * vpos(vR) + tr * vneg1(vR));
            dl += (double)nuR * (-(double)(tr - tc) * (double)a.idx[d]);
        }
    }
    a.gT(i, j, k) = g;
    if (a.has_gTold) a.gTold(i, j, k) = mc;
    return dl;
}

template <class T, int ND>
__global__ void __launch_bounds__(256) thermal_adjoint_kernel(const ThermalAdj<T> a) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int k = ND > 2 ? 1 + (int)blockIdx.z : 0;
    // every thread reaches the block sum once; threads beyond the grid add 0 to it
    double dl = 0.0;
    if (i <= a.n[0] && j <= a.n[1]) dl = thermal_adjoint_cell<T, ND>(a, i, j, k);
    block_sum_fixed(dl, a.gacc);
}

// Sum of `n` doubles in a fixed order (one block; see the diffusion adjoint's sum).
__global__ void __launch_bounds__(1024) thermal_sum_kernel(const double* __restrict__ x, long n, double* out) {
    __shared__ double part[1024];
    double s = 0.0;
    for (long q = threadIdx.x; q < n; q += 1024) s += x[q];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = part[0];
}

inline dim3 thermal_adjoint_block() { return dim3(32, 8); }
inline dim3 thermal_adjoint_grid(const cg_grid* g, dim3 b) {
    return dim3(cg_div_up(g->n[0], b.x), cg_div_up(g->n[1], b.y), g->ndim > 2 ? g->n[2] : 1);
}

template <class T, int ND>
int thermal_adjoint_t(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                      const int rule[3][2], const cg_field& mu, const cg_field& gT, const cg_field* gTold,
                      const cg_field* gV, double* gacc, double* sum) {
    ThermalAdj<T> a;
    std::memset(&a, 0, sizeof(a));
    a.Tin = cg_view<T>(f->T);
    a.mu = cg_view<T>(mu);
    a.gT = cg_view<T>(gT);
    a.has_gTold = gTold && gTold->data;
    if (a.has_gTold) a.gTold = cg_view<T>(*gTold);
    for (int d = 0; d < ND; ++d) {
        a.V[d] = cg_view<T>(f->V[d]);
        a.gV[d] = cg_view<T>(gV[d]);
        a.idx[d] = (T)g->inv_spacing[d];
        a.rule[d][0] = rule[d][0];
        a.rule[d][1] = rule[d][1];
    }
    for (int d = 0; d < 3; ++d) a.n[d] = d < ND ? g->n[d] : 1;
    a.lam = (T)p->lambda_rhoCp;
    a.dt = (T)p->dt;
    a.gacc = gacc;
    const dim3 b = thermal_adjoint_block();
    const dim3 grid = thermal_adjoint_grid(g, b);
    thermal_adjoint_kernel<T, ND><<<grid, b, 0, ctx->stream>>>(a);
    CG_CHECK_LAUNCH(ctx);
    if (sum) {
        thermal_sum_kernel<<<1, 1024, 0, ctx->stream>>>(gacc, (long)grid.x * grid.y * grid.z, sum);
        CG_CHECK_LAUNCH(ctx);
    }
    return CG_OK;
}

}  // namespace

extern "C" int cg_stokes_thermal_step_adjoint(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                              const cg_stokes_params* p, const cg_bc* bc_T, const cg_field* mu,
                                              const cg_field* gT, const cg_field* gT_old, const cg_field* gV,
                                              double* dJ) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_stokes_thermal_step_adjoint: ctx is NULL");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!f || !p || !bc_T || !mu || !gT || !gV)
        return cg_fail(ctx, CG_ERR_ARG, "cg_stokes_thermal_step_adjoint: NULL argument");
    const int nd = grid->ndim;
    if (nd < 2) return cg_fail(ctx, CG_ERR_ARG, "cg_stokes_thermal_step_adjoint: 2D or 3D grids only");
    const int dtype = f->T.dtype;
    if (dtype != CG_F32 && dtype != CG_F64) return cg_fail(ctx, CG_ERR_ARG, "cg_stokes_thermal_step_adjoint: bad dtype");
    if ((rc = cg_check_field(ctx, grid, f->T, dtype, 0, "T"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *mu, dtype, 0, "mu"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *gT, dtype, 0, "gT"))) return rc;
    if (gT_old && gT_old->data && (rc = cg_check_field(ctx, grid, *gT_old, dtype, 0, "gT_old"))) return rc;
    for (int d = 0; d < nd; ++d) {
        if ((rc = cg_check_field(ctx, grid, f->V[d], dtype, 1 << d, "V"))) return rc;
        if ((rc = cg_check_field(ctx, grid, gV[d], dtype, 1 << d, "gV"))) return rc;
    }
    int rule[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int d = 0; d < nd; ++d)
        for (int s = 0; s < 2; ++s) {
            const int kd = bc_T->kind[d][s];
            if (kd == CG_BC_NEUMANN) rule[d][s] = 1;
            else if (kd == CG_BC_DIRICHLET) rule[d][s] = -1;
            else if (kd == CG_BC_PERIODIC) rule[d][s] = 2;
            else
                return cg_fail(ctx, CG_ERR_UNSUPPORTED,
                               "cg_stokes_thermal_step_adjoint: side %d of dim %d of bc_T has no Dirichlet, Neumann or "
                               "Periodic rule", s, d);
        }
    cudaSetDevice(ctx->device);
    const dim3 tg = thermal_adjoint_grid(grid, thermal_adjoint_block());
    const long nblocks = (long)tg.x * tg.y * tg.z;
    double* gacc = static_cast<double*>(cg_scratch(ctx, kThermalSlot, (size_t)(nblocks + 32) * sizeof(double), &rc));
    if (rc) return rc;
    double* sum = dJ ? gacc + nblocks : nullptr;
    rc = dtype == CG_F64 ? (nd == 2 ? thermal_adjoint_t<double, 2>(ctx, grid, f, p, rule, *mu, *gT, gT_old, gV, gacc, sum)
                                    : thermal_adjoint_t<double, 3>(ctx, grid, f, p, rule, *mu, *gT, gT_old, gV, gacc, sum))
                         : (nd == 2 ? thermal_adjoint_t<float, 2>(ctx, grid, f, p, rule, *mu, *gT, gT_old, gV, gacc, sum)
                                    : thermal_adjoint_t<float, 3>(ctx, grid, f, p, rule, *mu, *gT, gT_old, gV, gacc, sum));
    if (rc) return rc;
    if (dJ) {
        double total = 0.0;
        CG_CUDA(ctx, cudaMemcpyAsync(&total, sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        dJ[0] += total;
    }
    return CG_OK;
}
