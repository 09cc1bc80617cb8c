// cg_diffusion_adjoint.cu — reverse time stepping of the explicit diffusion loop
// (examples/diffusion_2d.jl:8-19, time loop :44-47): a taped forward run and the reverse sweep.
//
// One step of the loop is C' = bc!(S C): S is the fused flux + update stencil of
// cg_diffusion_step (C' = C - dt divg(-chi grad C) over [0, n+1]^N) and bc! rewrites the ghost
// planes from the interior. Seen on the interior cells, the step is affine: the ghost value
// beside a boundary cell is alpha * C[cell] + const (Neumann alpha = +1, Center Dirichlet
// alpha = -1: f[g] = 2a - f[in]), or the opposite interior cell (Periodic). Its transpose is the
// same 5-point (7-point in 3D) stencil in gather form, with the neighbour beyond a side replaced
// by alpha * lambda[cell] or the wrapped cell, so the reverse step has the forward's cost:
//   lambda^n[I] = lambda[I] + sum_d a_d (lambda_r + lambda_l - 2 lambda[I]),  a_d = dt chi / dx_d^2
// with lambda = lambda^{n+1}. The step depends on chi through a_d only: dC^{n+1}[I]/dchi =
// (C^{n+1}[I] - C^n[I]) / chi at an interior cell, so dJ/dchi = (1/chi) sum_n sum_I
// lambda^{n+1}[I] (C^{n+1}[I] - C^n[I]), accumulated per cell in FP64 over the sweep and summed
// once, in a fixed order, at its end. The tape is the sequence of states C^0 .. C^N, which the
// forward run writes anyway.
#include "cg_common.cuh"

namespace {

constexpr unsigned long long kDiffTapeMagic = 0x4364696666546170ull;  // "CdiffTap"
constexpr int kGaccSlot = 8;  // ctx scratch slot: per-cell dJ/dchi sums and the final sum

struct DiffTapeHeader {
    unsigned long long magic;
    int dtype, ndim, nsteps, pad;
    int n[3], halo[3];
    long long stride[3];
    long long state_bytes;
    double chi, dt;
    int kind[3][2];
};
static_assert(sizeof(DiffTapeHeader) <= 256, "the tape header fits its 256 bytes");

// Elements from the allocation start to one past the last padded element of a field.
inline long field_span(const cg_field& f) {
    long span = 1;
    for (int d = 0; d < f.ndim; ++d) span += (long)(f.n[d] + 4 * f.halo[d] - 1) * f.stride[d];
    return span;
}

inline size_t state_bytes_of(const cg_field& f) {
    const size_t esz = f.dtype == CG_F64 ? 8 : 4;
    return ((size_t)field_span(f) * esz + 255) / 256 * 256;
}

inline cg_field state_field(const cg_field& like, const void* tape, int s) {
    cg_field f = like;
    f.data = const_cast<char*>(static_cast<const char*>(tape)) + 256 + (size_t)s * state_bytes_of(like);
    return f;
}

// How a side's ghost value follows from the interior: +1 Neumann, -1 Dirichlet (Center field),
// 2 Periodic (the opposite interior cell).
struct SideRule {
    int r[3][2];
};

inline int side_rules(cg_ctx* ctx, const cg_grid* g, const cg_bc* bc, SideRule* out) {
    for (int d = 0; d < 3; ++d)
        for (int s = 0; s < 2; ++s) {
            if (d >= g->ndim) {
                out->r[d][s] = 0;
                continue;
            }
            const int k = bc->kind[d][s];
            if (k == CG_BC_NEUMANN) out->r[d][s] = 1;
            else if (k == CG_BC_DIRICHLET) out->r[d][s] = -1;
            else if (k == CG_BC_PERIODIC) out->r[d][s] = 2;
            else
                return cg_fail(ctx, CG_ERR_UNSUPPORTED,
                               "diffusion adjoint: side %d of dim %d has no Dirichlet, Neumann or Periodic rule "
                               "(its ghost cell would be a state of its own)", s, d);
        }
    return CG_OK;
}

template <class T>
struct Coef {
    T a[3];
};

// lambda beyond side s of dim d of cell I, from the side's rule
template <class T>
__device__ __forceinline__ T beyond(const DF<T>& l, T lc, int rule, int d, int i, int j, int k, int nd_last) {
    if (rule == 2) {  // periodic: the opposite interior cell
        int I[3] = {i, j, k};
        I[d] = nd_last;
        return l(I[0], I[1], I[2]);
    }
    return rule > 0 ? lc : -lc;
}

// One reverse step over the interior cells [1, n]^N (gather form; no two threads write one
// address). gacc (dense n0 x n1 x n2, FP64) gains lambda (C^{n+1} - C^n) per cell.
template <class T, int ND>
__global__ void diffusion_adjoint_kernel(DF<T> lo, DF<T> li, DF<T> Cn, DF<T> Cn1, double* __restrict__ gacc,
                                         Coef<T> c, SideRule rule, int n0, int n1, int n2) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = ND > 1 ? 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y) : 0;
    const int k = ND > 2 ? 1 + (int)blockIdx.z : 0;
    if (i > n0 || (ND > 1 && j > n1)) return;
    const T l = li(i, j, k);
    // neighbours along x
    const T xl = i > 1 ? li(i - 1, j, k) : beyond(li, l, rule.r[0][0], 0, i, j, k, n0);
    const T xr = i < n0 ? li(i + 1, j, k) : beyond(li, l, rule.r[0][1], 0, i, j, k, 1);
    T acc = c.a[0] * fma(T(-2), l, xr + xl);
    if (ND > 1) {
        const T yl = j > 1 ? li(i, j - 1, k) : beyond(li, l, rule.r[1][0], 1, i, j, k, n1);
        const T yr = j < n1 ? li(i, j + 1, k) : beyond(li, l, rule.r[1][1], 1, i, j, k, 1);
        acc = fma(c.a[1], fma(T(-2), l, yr + yl), acc);
    }
    if (ND > 2) {
        const T zl = k > 1 ? li(i, j, k - 1) : beyond(li, l, rule.r[2][0], 2, i, j, k, n2);
        const T zr = k < n2 ? li(i, j, k + 1) : beyond(li, l, rule.r[2][1], 2, i, j, k, 1);
        acc = fma(c.a[2], fma(T(-2), l, zr + zl), acc);
    }
    lo(i, j, k) = l + acc;
    const long q = (long)(i - 1) + (long)n0 * ((ND > 1 ? (long)(j - 1) : 0) + (long)n1 * (ND > 2 ? (long)(k - 1) : 0));
    gacc[q] = fma((double)l, (double)Cn1(i, j, k) - (double)Cn(i, j, k), gacc[q]);
}

// Sum of `n` doubles in a fixed order: one block of 1024 threads, thread t adds elements
// t, t + 1024, ... in turn, then a fixed tree over the threads.
__global__ void __launch_bounds__(1024) fixed_order_sum_kernel(const double* __restrict__ x, long n, double* out) {
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

template <int ND>
inline dim3 interior_block() {
    return ND == 1 ? dim3(256, 1) : dim3(32, 8);
}

template <int ND>
inline dim3 interior_grid(const cg_grid* g, dim3 b) {
    return dim3(cg_div_up(g->n[0], b.x), ND > 1 ? cg_div_up(g->n[1], b.y) : 1, ND > 2 ? g->n[2] : 1);
}

template <class T, int ND>
int adjoint_step_t(cg_ctx* ctx, const cg_grid* g, const cg_field& lo, const cg_field& li, const cg_field& Cn,
                   const cg_field& Cn1, double* gacc, double chi, double dt, const SideRule& rule) {
    Coef<T> c;
    for (int d = 0; d < 3; ++d) c.a[d] = (T)(dt * chi * g->inv_spacing[d] * g->inv_spacing[d]);
    const dim3 b = interior_block<ND>();
    diffusion_adjoint_kernel<T, ND><<<interior_grid<ND>(g, b), b, 0, ctx->stream>>>(
        cg_view<T>(lo), cg_view<T>(li), cg_view<T>(Cn), cg_view<T>(Cn1), gacc, c, rule, g->n[0],
        ND > 1 ? g->n[1] : 1, ND > 2 ? g->n[2] : 1);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

#define CG_DISPATCH_ADJ(fn, dtype, nd, ...)                                                            \
    ((dtype) == CG_F64 ? ((nd) == 1 ? fn<double, 1>(__VA_ARGS__)                                      \
                                    : (nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__)) \
                       : ((nd) == 1 ? fn<float, 1>(__VA_ARGS__)                                       \
                                    : (nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

inline long interior_cells(const cg_grid* g) {
    long n = 1;
    for (int d = 0; d < g->ndim; ++d) n *= g->n[d];
    return n;
}

inline bool same_layout(const cg_field& a, const cg_field& b) {
    if (a.dtype != b.dtype || a.ndim != b.ndim) return false;
    for (int d = 0; d < a.ndim; ++d)
        if (a.n[d] != b.n[d] || a.halo[d] != b.halo[d] || a.stride[d] != b.stride[d] || a.loc[d] != b.loc[d])
            return false;
    return true;
}

DiffTapeHeader make_header(const cg_field& C, int nsteps, double chi, double dt, const cg_bc& bc) {
    DiffTapeHeader h;
    std::memset(&h, 0, sizeof(h));
    h.magic = kDiffTapeMagic;
    h.dtype = C.dtype;
    h.ndim = C.ndim;
    h.nsteps = nsteps;
    for (int d = 0; d < 3; ++d) {
        h.n[d] = C.n[d];
        h.halo[d] = C.halo[d];
        h.stride[d] = C.stride[d];
        for (int s = 0; s < 2; ++s) h.kind[d][s] = d < C.ndim ? bc.kind[d][s] : 0;
    }
    h.state_bytes = (long long)state_bytes_of(C);
    h.chi = chi;
    h.dt = dt;
    return h;
}

}  // namespace

extern "C" int cg_diffusion_tape_bytes(const cg_grid* grid, const cg_field* C, int nsteps, size_t* bytes) {
    if (!grid || !C || !bytes || nsteps < 0) return cg_fail(nullptr, CG_ERR_ARG, "cg_diffusion_tape_bytes: bad argument");
    *bytes = 256 + (size_t)(nsteps + 1) * state_bytes_of(*C);
    return CG_OK;
}

extern "C" int cg_diffusion_run_taped(cg_ctx* ctx, const cg_grid* grid, const cg_field* C, double chi, double dt,
                                      const cg_bc* bc, int nsteps, void* tape, size_t tape_bytes) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_diffusion_run_taped: ctx is NULL");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!C || !bc || !tape) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_taped: NULL argument");
    if ((rc = cg_check_field(ctx, grid, *C, C->dtype, 0, "C"))) return rc;
    if (C->dtype != CG_F32 && C->dtype != CG_F64) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_taped: bad dtype");
    if (nsteps < 1) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_taped: nsteps < 1");
    SideRule rule;
    if ((rc = side_rules(ctx, grid, bc, &rule))) return rc;
    size_t need = 0;
    cg_diffusion_tape_bytes(grid, C, nsteps, &need);
    if (tape_bytes < need) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_taped: tape of %zu bytes, %zu needed", tape_bytes, need);
    if (reinterpret_cast<uintptr_t>(tape) % 256) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_taped: tape not 256-byte aligned");
    cudaSetDevice(ctx->device);
    const DiffTapeHeader h = make_header(*C, nsteps, chi, dt, *bc);
    const size_t esz = C->dtype == CG_F64 ? 8 : 4;
    const size_t span = (size_t)field_span(*C) * esz;
    // the header from pageable memory: the copy is staged before the call returns
    CG_CUDA(ctx, cudaMemcpyAsync(tape, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    const cg_field s0 = state_field(*C, tape, 0);
    CG_CUDA(ctx, cudaMemcpyAsync(s0.data, C->data, span, cudaMemcpyDeviceToDevice, ctx->stream));
    std::string key = "diffusion_run_taped";
    cg_key_add(key, *grid);
    cg_key_add(key, *C);
    cg_key_add(key, chi);
    cg_key_add(key, dt);
    cg_key_add(key, nsteps);
    cg_key_add(key, *bc);
    cg_key_add(key, tape);
    // the last step writes the caller's field, which so keeps its own outer halo (the layer no
    // step writes) as the in-place loop does; its result is then recorded as state nsteps
    rc = cg_graph_run(ctx, key, [&](cudaStream_t) {
        for (int s = 0; s < nsteps; ++s) {
            const cg_field in = state_field(*C, tape, s);
            const cg_field out = s + 1 < nsteps ? state_field(*C, tape, s + 1) : *C;
            int r = cg_diffusion_step(ctx, grid, &out, &in, chi, dt, bc);
            if (r) return r;
        }
        return (int)CG_OK;
    });
    if (rc) return rc;
    const cg_field sN = state_field(*C, tape, nsteps);
    CG_CUDA(ctx, cudaMemcpyAsync(sN.data, C->data, span, cudaMemcpyDeviceToDevice, ctx->stream));
    return CG_OK;
}

extern "C" int cg_diffusion_adjoint_run(cg_ctx* ctx, const cg_grid* grid, const void* tape, size_t tape_bytes,
                                        const cg_field* lam, const cg_field* work, double chi, double dt,
                                        const cg_bc* bc, double* dJ) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_diffusion_adjoint_run: ctx is NULL");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!tape || !lam || !work || !bc) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: NULL argument");
    if ((rc = cg_check_field(ctx, grid, *lam, lam->dtype, 0, "lam"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *work, lam->dtype, 0, "work"))) return rc;
    if (!same_layout(*lam, *work)) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: work must have lam's layout");
    if (lam->data == work->data) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: work aliases lam");
    if (tape_bytes < 256) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: tape too small");
    SideRule rule;
    if ((rc = side_rules(ctx, grid, bc, &rule))) return rc;
    cudaSetDevice(ctx->device);
    DiffTapeHeader h;
    CG_CUDA(ctx, cudaMemcpyAsync(&h, tape, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const DiffTapeHeader want = make_header(*lam, h.nsteps, chi, dt, *bc);
    if (h.magic != kDiffTapeMagic || h.nsteps < 1)
        return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: not a tape of cg_diffusion_run_taped");
    if (std::memcmp(&h, &want, sizeof(h)) != 0)
        return cg_fail(ctx, CG_ERR_ARG,
                       "cg_diffusion_adjoint_run: lam's layout, chi, dt or the boundary kinds differ from the taped run's");
    const int nsteps = h.nsteps;
    size_t need = 0;
    cg_diffusion_tape_bytes(grid, lam, nsteps, &need);
    if (tape_bytes < need) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_adjoint_run: tape shorter than its %d steps", nsteps);
    const long ncell = interior_cells(grid);
    double* gacc = static_cast<double*>(cg_scratch(ctx, kGaccSlot, (size_t)(ncell + 32) * sizeof(double), &rc));
    if (rc) return rc;
    double* sum = gacc + ncell;
    CG_CUDA(ctx, cudaMemsetAsync(gacc, 0, (size_t)ncell * sizeof(double), ctx->stream));
    std::string key = "diffusion_adjoint_run";
    cg_key_add(key, *grid);
    cg_key_add(key, *lam);
    cg_key_add(key, *work);
    cg_key_add(key, chi);
    cg_key_add(key, dt);
    cg_key_add(key, *bc);
    cg_key_add(key, tape);
    cg_key_add(key, gacc);
    cg_key_add(key, nsteps);
    rc = cg_graph_run(ctx, key, [&](cudaStream_t) {
        for (int s = nsteps - 1, q = 0; s >= 0; --s, ++q) {
            const cg_field& in = (q % 2 == 0) ? *lam : *work;
            const cg_field& out = (q % 2 == 0) ? *work : *lam;
            const cg_field Cn = state_field(*lam, tape, s), Cn1 = state_field(*lam, tape, s + 1);
            int r = CG_DISPATCH_ADJ(adjoint_step_t, lam->dtype, grid->ndim, ctx, grid, out, in, Cn, Cn1, gacc, chi, dt, rule);
            if (r) return r;
        }
        fixed_order_sum_kernel<<<1, 1024, 0, ctx->stream>>>(gacc, ncell, sum);
        CG_CHECK_LAUNCH(ctx);
        return (int)CG_OK;
    });
    if (rc) return rc;
    if (nsteps % 2 == 1) {  // the last reverse step wrote work
        const size_t span = (size_t)field_span(*lam) * (lam->dtype == CG_F64 ? 8 : 4);
        CG_CUDA(ctx, cudaMemcpyAsync(lam->data, work->data, span, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    double total = 0.0;
    CG_CUDA(ctx, cudaMemcpyAsync(&total, sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (dJ) dJ[0] += total / chi;
    return CG_OK;
}
