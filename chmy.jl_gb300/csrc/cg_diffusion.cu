// cg_diffusion.cu — explicit linear diffusion (Chmy.jl examples/diffusion_2d.jl:8-19).
#include "cg_common.cuh"


namespace {

using cgk::radd;
using cgk::rmul;
using cgk::rsub;

// Every kernel here rounds each operation as the oracle does (no contraction into FMA, the
// reference's operation order), so all of them equal the oracle bit for bit.

template <class T>
struct Spacing {
    T i[3];
};

// Threads cover the launcher range [0, n+1] in x and y; z (3D) is blockIdx.z. 1D launches use
// a flat block so that no two threads own the same point.
template <int ND>
inline dim3 block_for() {
    return ND == 1 ? dim3(256, 1) : dim3(32, 8);
}

template <int ND>
inline dim3 range_grid(const cg_grid* g, dim3 block) {
    return dim3(cg_div_up(g->n[0] + 2, block.x), ND > 1 ? cg_div_up(g->n[1] + 2, block.y) : 1,
                ND > 2 ? g->n[2] + 2 : 1);
}

template <class T, int ND>
__global__ void compute_q_kernel(DF<T> q0, DF<T> q1, DF<T> q2, DF<T> C, T mchi, Spacing<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const T c = C(i, j, k);
    // q.d = -χ * ∂d(C): C is Center, seen from the face: (C[I] - C[I - e_d]) * iΔ_d
    q0(i, j, k) = rmul(mchi, rmul(rsub(c, C(i - 1, j, k)), s.i[0]));
    if (ND > 1) q1(i, j, k) = rmul(mchi, rmul(rsub(c, C(i, j - 1, k)), s.i[1]));
    if (ND > 2) q2(i, j, k) = rmul(mchi, rmul(rsub(c, C(i, j, k - 1)), s.i[2]));
}

template <class T, int ND>
__global__ void update_C_kernel(DF<T> C, DF<T> q0, DF<T> q1, DF<T> q2, T dt, Spacing<T> s, int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    // divg(q) = Σ_d (q_d[I + e_d] - q_d[I]) * iΔ_d, summed in dim order
    T dv = rmul(rsub(q0(i + 1, j, k), q0(i, j, k)), s.i[0]);
    if (ND > 1) dv = radd(dv, rmul(rsub(q1(i, j + 1, k), q1(i, j, k)), s.i[1]));
    if (ND > 2) dv = radd(dv, rmul(rsub(q2(i, j, k + 1), q2(i, j, k)), s.i[2]));
    C(i, j, k) = rsub(C(i, j, k), rmul(dt, dv));
}

// Fused compute_q! + update_C! in the reference's flux form: q_d at face I is
// -χ ((C[I] - C[I-e_d]) iΔ_d) over the launch range, a face with index n+2 along its dimension is
// outside compute_q!'s range and reads as zero (fresh q arrays), and C' = C - dt Σ_d (q_d[I+e_d] -
// q_d[I]) iΔ_d in dim order. Each x-face flux is computed once (a lane's right face is the next
// lane's left face; the warp's last lane computes its own), each y-face once per block (row r of
// the block's shared array is the lower face of its row r), z-faces by both cells. Blocks are a
// multiple of 32 threads wide, so that a warp is 32 consecutive cells of one row.
template <class T, int ND>
__global__ void diffusion_step_kernel(DF<T> Co, DF<T> Ci, T mchi, T dt, Spacing<T> s, int e0, int e1, int e2) {
    extern __shared__ __align__(16) unsigned char dsm[];
    T* qy = reinterpret_cast<T*>(dsm);  // (blockDim.y + 1) x blockDim.x y-faces (2D, 3D)
    const int tx = threadIdx.x, ty = threadIdx.y, bx = blockDim.x;
    const int i = blockIdx.x * bx + tx;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + ty : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    const bool in = i <= e0 && j <= e1;
    auto face = [&](T a, T b, int d) { return rmul(mchi, rmul(rsub(a, b), s.i[d])); };
    T c = T(0), qxl = T(0);
    if (in) {
        c = Ci(i, j, k);
        qxl = face(c, Ci(i - 1, j, k), 0);
    }
    T qxr = __shfl_down_sync(0xffffffffu, qxl, 1);
    if ((tx & 31) == 31) qxr = (in && i + 1 <= e0) ? face(Ci(i + 1, j, k), c, 0) : T(0);
    T qyl = T(0), qyr = T(0);
    if constexpr (ND > 1) {
        qy[ty * bx + tx] = in ? face(c, Ci(i, j - 1, k), 1) : T(0);
        if (ty == (int)blockDim.y - 1) qy[(ty + 1) * bx + tx] = (in && j + 1 <= e1) ? face(Ci(i, j + 1, k), c, 1) : T(0);
        __syncthreads();
        qyl = qy[ty * bx + tx];
        qyr = qy[(ty + 1) * bx + tx];
    }
    if (!in) return;
    T dv = rmul(rsub(qxr, qxl), s.i[0]);
    if constexpr (ND > 1) dv = radd(dv, rmul(rsub(qyr, qyl), s.i[1]));
    if constexpr (ND > 2) {
        const T qzl = face(c, Ci(i, j, k - 1), 2);
        const T qzr = k + 1 <= e2 ? face(Ci(i, j, k + 1), c, 2) : T(0);
        dv = radd(dv, rmul(rsub(qzr, qzl), s.i[2]));
    }
    Co(i, j, k) = rsub(c, rmul(dt, dv));
}

// ---- masked operators (src/GridOperators/masked_operators.jl:11-39) --------------------------
// A masked operator multiplies every operand value by the mask at the operand's location and
// index: the masked ∂_d of Center C at face I is (C[I] w_c[I] - C[I-e_d] w_c[I-e_d]) iΔ_d, and
// the masked divg of q is Σ_d (q_d[I+e_d] w_d[I+e_d] - q_d[I] w_d[I]) iΔ_d (masked_field_
// operators.jl:52-57). w_c is the Center mask, w_d the mask at the d-face location (Vertex
// along d).
template <class T>
struct MaskV {
    DF<T> c, f[3];
};

template <class T, int ND>
__global__ void compute_q_masked_kernel(DF<T> q0, DF<T> q1, DF<T> q2, DF<T> C, const MaskV<T> w, T mchi, Spacing<T> s,
                                        int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const T cw = rmul(C(i, j, k), w.c(i, j, k));
    q0(i, j, k) = rmul(mchi, rmul(rsub(cw, rmul(C(i - 1, j, k), w.c(i - 1, j, k))), s.i[0]));
    if (ND > 1) q1(i, j, k) = rmul(mchi, rmul(rsub(cw, rmul(C(i, j - 1, k), w.c(i, j - 1, k))), s.i[1]));
    if (ND > 2) q2(i, j, k) = rmul(mchi, rmul(rsub(cw, rmul(C(i, j, k - 1), w.c(i, j, k - 1))), s.i[2]));
}

template <class T, int ND>
__global__ void update_C_masked_kernel(DF<T> C, DF<T> q0, DF<T> q1, DF<T> q2, const MaskV<T> w, T dt, Spacing<T> s,
                                       int e0, int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    T dv = rmul(rsub(rmul(q0(i + 1, j, k), w.f[0](i + 1, j, k)), rmul(q0(i, j, k), w.f[0](i, j, k))), s.i[0]);
    if (ND > 1)
        dv = radd(dv, rmul(rsub(rmul(q1(i, j + 1, k), w.f[1](i, j + 1, k)), rmul(q1(i, j, k), w.f[1](i, j, k))), s.i[1]));
    if (ND > 2)
        dv = radd(dv, rmul(rsub(rmul(q2(i, j, k + 1), w.f[2](i, j, k + 1)), rmul(q2(i, j, k), w.f[2](i, j, k))), s.i[2]));
    C(i, j, k) = rsub(C(i, j, k), rmul(dt, dv));
}

// Fused masked compute_q! + update_C! (a flux at index n+2 reads as zero, as in the unmasked
// fused step)
template <class T, int ND>
__global__ void diffusion_step_masked_kernel(DF<T> Co, DF<T> Ci, const MaskV<T> w, T mchi, T dt, Spacing<T> s, int e0,
                                             int e1, int e2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = ND > 1 ? blockIdx.y * blockDim.y + threadIdx.y : 0;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const T c = Ci(i, j, k);
    const T cw = rmul(c, w.c(i, j, k));
    const int I[3] = {i, j, k}, E[3] = {e0, e1, e2};
    T dv = T(0);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const int di = d == 0, dj = d == 1, dk = d == 2;
        const T ql = rmul(mchi, rmul(rsub(cw, rmul(Ci(i - di, j - dj, k - dk), w.c(i - di, j - dj, k - dk))), s.i[d]));
        const T qr = I[d] + 1 <= E[d]
                         ? rmul(mchi, rmul(rsub(rmul(Ci(i + di, j + dj, k + dk), w.c(i + di, j + dj, k + dk)), cw), s.i[d]))
                         : T(0);
        const T t = rmul(rsub(rmul(qr, w.f[d](i + di, j + dj, k + dk)), rmul(ql, w.f[d](i, j, k))), s.i[d]);
        dv = d == 0 ? t : radd(dv, t);
    }
    Co(i, j, k) = rsub(c, rmul(dt, dv));
}

template <class T>
Spacing<T> spacing_of(const cg_grid* g) {
    Spacing<T> s;
    for (int d = 0; d < 3; ++d) s.i[d] = (T)g->inv_spacing[d];
    return s;
}

int check_q(cg_ctx* ctx, const cg_grid* grid, const cg_field* q, int dtype) {
    for (int d = 0; d < grid->ndim; ++d) {
        int rc = cg_check_field(ctx, grid, q[d], dtype, 1 << d, "q");
        if (rc) return rc;
    }
    return CG_OK;
}

template <class T, int ND>
int compute_q_t(cg_ctx* ctx, const cg_grid* g, const cg_field* q, const cg_field* C, double chi) {
    const dim3 block = block_for<ND>();
    DF<T> Q[3] = {cg_view<T>(q[0]), ND > 1 ? cg_view<T>(q[1]) : DF<T>{}, ND > 2 ? cg_view<T>(q[2]) : DF<T>{}};
    compute_q_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        Q[0], Q[1], Q[2], cg_view<T>(*C), -(T)chi, spacing_of<T>(g), g->n[0] + 1, ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int update_C_t(cg_ctx* ctx, const cg_grid* g, const cg_field* C, const cg_field* q, double dt) {
    const dim3 block = block_for<ND>();
    DF<T> Q[3] = {cg_view<T>(q[0]), ND > 1 ? cg_view<T>(q[1]) : DF<T>{}, ND > 2 ? cg_view<T>(q[2]) : DF<T>{}};
    update_C_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        cg_view<T>(*C), Q[0], Q[1], Q[2], (T)dt, spacing_of<T>(g), g->n[0] + 1, ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
cudaError_t step_launch(const cg_grid* g, const cg_field* Co, const cg_field* Ci, double chi, double dt, dim3 block,
                        cudaStream_t st) {
    const size_t smem = ND > 1 ? (size_t)(block.y + 1) * block.x * sizeof(T) : 0;
    diffusion_step_kernel<T, ND><<<range_grid<ND>(g, block), block, smem, st>>>(
        cg_view<T>(*Co), cg_view<T>(*Ci), -(T)chi, (T)dt, spacing_of<T>(g), g->n[0] + 1,
        ND > 1 ? g->n[1] + 1 : 0, ND > 2 ? g->n[2] + 1 : 0);
    return cudaGetLastError();
}

// The step kernel's block shape for this grid and layout: 1D keeps 256 threads; 2D and 3D take
// the autotuner's choice, timed on C_out = step(C_in) (the first step of a run writes the same
// points again), or its cached choice when `may_time` is false.
template <class T, int ND>
dim3 step_block(cg_ctx* ctx, const cg_grid* g, const cg_field* Co, const cg_field* Ci, double chi, double dt,
                bool may_time) {
    if (ND == 1) return block_for<ND>();
    std::string key = "diffusion_block";
    cg_key_add(key, *g);
    cg_key_add(key, (int)sizeof(T));
    cg_key_add(key, Ci->stride);
    cg_key_add(key, Co->stride);
    cg_key_add(key, ctx->num_sms);
    if (!may_time) {
        dim3 b(32, 8);
        if (cg_block_forced(&b)) return b;
        cg_tune_cfg c{0, 0};
        return cg_tune_lookup(key, &c) ? dim3((unsigned)c.seg, (unsigned)c.variant) : b;
    }
    return cgk::tune_block("diffusion step", key,
                           [&](dim3 b) { return step_launch<T, ND>(g, Co, Ci, chi, dt, b, ctx->stream); }, ctx->stream);
}

template <class T, int ND>
int step_t(cg_ctx* ctx, const cg_grid* g, const cg_field* Co, const cg_field* Ci, double chi, double dt, bool may_time) {
    const dim3 block = step_block<T, ND>(ctx, g, Co, Ci, chi, dt, may_time);
    const cudaError_t e = step_launch<T, ND>(g, Co, Ci, chi, dt, block, ctx->stream);
    if (e != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "diffusion step: %s", cudaGetErrorString(e));
    return CG_OK;
}

template <class T>
MaskV<T> mask_view(const cg_mask* m, int nd) {
    MaskV<T> w;
    std::memset(&w, 0, sizeof(w));
    w.c = cg_view<T>(m->at[0]);
    for (int d = 0; d < nd; ++d) w.f[d] = cg_view<T>(m->at[1 << d]);
    return w;
}

template <class T, int ND>
int compute_q_masked_t(cg_ctx* ctx, const cg_grid* g, const cg_field* q, const cg_field* C, double chi, const cg_mask* m) {
    const dim3 block = block_for<ND>();
    DF<T> Q[3] = {cg_view<T>(q[0]), ND > 1 ? cg_view<T>(q[1]) : DF<T>{}, ND > 2 ? cg_view<T>(q[2]) : DF<T>{}};
    compute_q_masked_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        Q[0], Q[1], Q[2], cg_view<T>(*C), mask_view<T>(m, ND), -(T)chi, spacing_of<T>(g), g->n[0] + 1,
        ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int update_C_masked_t(cg_ctx* ctx, const cg_grid* g, const cg_field* C, const cg_field* q, double dt, const cg_mask* m) {
    const dim3 block = block_for<ND>();
    DF<T> Q[3] = {cg_view<T>(q[0]), ND > 1 ? cg_view<T>(q[1]) : DF<T>{}, ND > 2 ? cg_view<T>(q[2]) : DF<T>{}};
    update_C_masked_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        cg_view<T>(*C), Q[0], Q[1], Q[2], mask_view<T>(m, ND), (T)dt, spacing_of<T>(g), g->n[0] + 1,
        ND > 1 ? g->n[1] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

template <class T, int ND>
int step_masked_t(cg_ctx* ctx, const cg_grid* g, const cg_field* Co, const cg_field* Ci, double chi, double dt,
                  const cg_mask* m) {
    const dim3 block = block_for<ND>();
    diffusion_step_masked_kernel<T, ND><<<range_grid<ND>(g, block), block, 0, ctx->stream>>>(
        cg_view<T>(*Co), cg_view<T>(*Ci), mask_view<T>(m, ND), -(T)chi, (T)dt, spacing_of<T>(g), g->n[0] + 1,
        ND > 1 ? g->n[1] + 1 : 0, ND > 2 ? g->n[2] + 1 : 0);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// The mask entries the diffusion kernels read: Center and the ndim face locations.
int check_mask(cg_ctx* ctx, const cg_grid* grid, const cg_mask* m, int dtype) {
    if (!m) return cg_fail(ctx, CG_ERR_ARG, "masked diffusion: NULL mask");
    int rc = cg_check_field(ctx, grid, m->at[0], dtype, 0, "mask (Center)");
    if (rc) return rc;
    for (int d = 0; d < grid->ndim; ++d)
        if ((rc = cg_check_field(ctx, grid, m->at[1 << d], dtype, 1 << d, "mask (face)"))) return rc;
    return CG_OK;
}

}  // namespace

#define CG_DISPATCH(fn, dtype, nd, ...)                                                              \
    ((dtype) == CG_F64 ? ((nd) == 1 ? fn<double, 1>(__VA_ARGS__)                                    \
                                    : (nd) == 2 ? fn<double, 2>(__VA_ARGS__) : fn<double, 3>(__VA_ARGS__)) \
                       : ((nd) == 1 ? fn<float, 1>(__VA_ARGS__)                                     \
                                    : (nd) == 2 ? fn<float, 2>(__VA_ARGS__) : fn<float, 3>(__VA_ARGS__)))

extern "C" int cg_diffusion_compute_q(cg_ctx* ctx, const cg_grid* grid, const cg_field* q, const cg_field* C,
                                      double chi) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!q || !C) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_compute_q: NULL field");
    cudaSetDevice(ctx->device);
    if ((rc = cg_check_field(ctx, grid, *C, C->dtype, 0, "C"))) return rc;
    if ((rc = check_q(ctx, grid, q, C->dtype))) return rc;
    return CG_DISPATCH(compute_q_t, C->dtype, grid->ndim, ctx, grid, q, C, chi);
}

extern "C" int cg_diffusion_update_C(cg_ctx* ctx, const cg_grid* grid, const cg_field* C, const cg_field* q,
                                     double dt) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!q || !C) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_update_C: NULL field");
    cudaSetDevice(ctx->device);
    if ((rc = cg_check_field(ctx, grid, *C, C->dtype, 0, "C"))) return rc;
    if ((rc = check_q(ctx, grid, q, C->dtype))) return rc;
    return CG_DISPATCH(update_C_t, C->dtype, grid->ndim, ctx, grid, C, q, dt);
}

// One step and bc!; `may_time`: the block-shape autotuner may time launches (false inside a
// graph capture, where the cached or default shape is used).
static int step_checked(cg_ctx* ctx, const cg_grid* grid, const cg_field* Co, const cg_field* Ci, double chi,
                        double dt, const cg_bc* bc, bool may_time) {
    int rc = CG_DISPATCH(step_t, Ci->dtype, grid->ndim, ctx, grid, Co, Ci, chi, dt, may_time);
    if (rc) return rc;
    if (bc) return cg_bc_apply_impl(ctx, grid, 1, Co, bc);
    return CG_OK;
}

static int step_args(cg_ctx* ctx, const cg_grid* grid, const cg_field* Co, const cg_field* Ci) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!Co || !Ci) return cg_fail(ctx, CG_ERR_ARG, "diffusion step: NULL field");
    if ((rc = cg_check_field(ctx, grid, *Ci, Ci->dtype, 0, "C_in"))) return rc;
    if ((rc = cg_check_field(ctx, grid, *Co, Ci->dtype, 0, "C_out"))) return rc;
    if (Co->data == Ci->data) return cg_fail(ctx, CG_ERR_ARG, "diffusion step: C_out aliases C_in");
    return CG_OK;
}

extern "C" int cg_diffusion_step(cg_ctx* ctx, const cg_grid* grid, const cg_field* C_out, const cg_field* C_in,
                                 double chi, double dt, const cg_bc* bc) {
    int rc = step_args(ctx, grid, C_out, C_in);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    return step_checked(ctx, grid, C_out, C_in, chi, dt, bc, false);
}

extern "C" int cg_diffusion_run(cg_ctx* ctx, const cg_grid* grid, const cg_field* A, const cg_field* B, double chi,
                                double dt, const cg_bc* bc, int nsteps) {
    int rc = step_args(ctx, grid, B, A);
    if (rc) return rc;
    if (nsteps < 0) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run: nsteps < 0");
    if (nsteps == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    std::string key = "diffusion_run";
    cg_key_add(key, *grid);
    cg_key_add(key, *A);
    cg_key_add(key, *B);
    cg_key_add(key, chi);
    cg_key_add(key, dt);
    cg_key_add(key, nsteps);
    cg_bc none;
    std::memset(&none, 0, sizeof(none));
    cg_key_add(key, bc ? *bc : none);
    // the step's block shape, timed on B = step(A) (once per shape) before the graph is captured
    dim3 blk(256, 1);
    if (grid->ndim > 1) blk = A->dtype == CG_F64
                                  ? (grid->ndim == 2 ? step_block<double, 2>(ctx, grid, B, A, chi, dt, true)
                                                     : step_block<double, 3>(ctx, grid, B, A, chi, dt, true))
                                  : (grid->ndim == 2 ? step_block<float, 2>(ctx, grid, B, A, chi, dt, true)
                                                     : step_block<float, 3>(ctx, grid, B, A, chi, dt, true));
    cg_key_add(key, blk);
    return cg_graph_run(ctx, key, [&](cudaStream_t) {
        for (int s = 0; s < nsteps; ++s) {
            const cg_field* in = (s % 2 == 0) ? A : B;
            const cg_field* out = (s % 2 == 0) ? B : A;
            int r = step_checked(ctx, grid, out, in, chi, dt, bc, false);
            if (r) return r;
        }
        return (int)CG_OK;
    });
}

// ---- masked forms -------------------------------------------------------------------------

extern "C" int cg_diffusion_compute_q_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* q, const cg_field* C,
                                             double chi, const cg_mask* mask) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!q || !C) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_compute_q_masked: NULL field");
    cudaSetDevice(ctx->device);
    if ((rc = cg_check_field(ctx, grid, *C, C->dtype, 0, "C"))) return rc;
    if ((rc = check_q(ctx, grid, q, C->dtype))) return rc;
    if ((rc = check_mask(ctx, grid, mask, C->dtype))) return rc;
    return CG_DISPATCH(compute_q_masked_t, C->dtype, grid->ndim, ctx, grid, q, C, chi, mask);
}

extern "C" int cg_diffusion_update_C_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* C, const cg_field* q,
                                            double dt, const cg_mask* mask) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!q || !C) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_update_C_masked: NULL field");
    cudaSetDevice(ctx->device);
    if ((rc = cg_check_field(ctx, grid, *C, C->dtype, 0, "C"))) return rc;
    if ((rc = check_q(ctx, grid, q, C->dtype))) return rc;
    if ((rc = check_mask(ctx, grid, mask, C->dtype))) return rc;
    return CG_DISPATCH(update_C_masked_t, C->dtype, grid->ndim, ctx, grid, C, q, dt, mask);
}

extern "C" int cg_diffusion_run_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* A, const cg_field* B,
                                       double chi, double dt, const cg_bc* bc, const cg_mask* mask, int nsteps) {
    int rc = step_args(ctx, grid, B, A);
    if (rc) return rc;
    if (nsteps < 0) return cg_fail(ctx, CG_ERR_ARG, "cg_diffusion_run_masked: nsteps < 0");
    if ((rc = check_mask(ctx, grid, mask, A->dtype))) return rc;
    if (nsteps == 0) return CG_OK;
    cudaSetDevice(ctx->device);
    std::string key = "diffusion_run_masked";
    cg_key_add(key, *grid);
    cg_key_add(key, *A);
    cg_key_add(key, *B);
    cg_key_add(key, *mask);
    cg_key_add(key, chi);
    cg_key_add(key, dt);
    cg_key_add(key, nsteps);
    cg_bc none;
    std::memset(&none, 0, sizeof(none));
    cg_key_add(key, bc ? *bc : none);
    return cg_graph_run(ctx, key, [&](cudaStream_t) {
        for (int s = 0; s < nsteps; ++s) {
            const cg_field* in = (s % 2 == 0) ? A : B;
            const cg_field* out = (s % 2 == 0) ? B : A;
            int r = CG_DISPATCH(step_masked_t, in->dtype, grid->ndim, ctx, grid, out, in, chi, dt, mask);
            if (r) return r;
            if (bc && (r = cg_bc_apply_impl(ctx, grid, 1, out, bc))) return r;
        }
        return (int)CG_OK;
    });
}
