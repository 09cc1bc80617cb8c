// cg_function.cu — device FunctionFields (src/Fields/function_field.jl:49-59): set!(f, grid, func)
// evaluated on the device for the function forms the kernels know (cg_function).
#include "cg_stokes_kernels.cuh"

namespace {

template <class T, int ND>
__global__ void function_fill_kernel(DF<T> f, cgk::FnDev<T> fn, T org0, T org1, T org2, T dx0, T dx1, T dx2, int v0,
                                     int v1, int v2, int lo0, int lo1, int lo2, int ext0, int ext1) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y * blockDim.y + threadIdx.y;
    const int c = blockIdx.z;
    if (a >= ext0 || b >= ext1) return;
    const int i = lo0 + a, j = ND > 1 ? lo1 + b : 0, k = ND > 2 ? lo2 + c : 0;
    T x[3] = {T(0), T(0), T(0)};
    x[0] = cgk::grid_coord(org0, dx0, i, v0 != 0);
    if (ND > 1) x[1] = cgk::grid_coord(org1, dx1, j, v1 != 0);
    if (ND > 2) x[2] = cgk::grid_coord(org2, dx2, k, v2 != 0);
    f(i, j, k) = cgk::fn_eval(fn, ND, x);
}

template <class T, int ND>
int fill_t(cg_ctx* ctx, const cg_grid* g, const cg_function* fn, const cg_field& f) {
    cgk::FnDev<T> d;
    d.kind = fn->kind;
    for (int q = 0; q < 8; ++q) d.p[q] = (T)fn->p[q];
    int lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
    for (int e = 0; e < ND; ++e) {
        lo[e] = 1 - 2 * f.halo[e];
        ext[e] = f.n[e] + 4 * f.halo[e];
    }
    const dim3 b(32, 8);
    const dim3 grid(cg_div_up(ext[0], b.x), cg_div_up(ext[1], b.y), ext[2]);
    function_fill_kernel<T, ND><<<grid, b, 0, ctx->stream>>>(
        cg_view<T>(f), d, (T)g->origin[0], (T)g->origin[1], (T)g->origin[2], (T)g->spacing[0], (T)g->spacing[1],
        (T)g->spacing[2], f.loc[0], ND > 1 ? f.loc[1] : 0, ND > 2 ? f.loc[2] : 0, lo[0], lo[1], lo[2], ext[0], ext[1]);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

}  // namespace

extern "C" int cg_function_fill(cg_ctx* ctx, const cg_grid* grid, const cg_function* fn, const cg_field* f) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_function_fill: ctx is NULL");
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (!fn || !f) return cg_fail(ctx, CG_ERR_ARG, "cg_function_fill: NULL argument");
    if (fn->kind < CG_FN_CONST || fn->kind > CG_FN_AFFINE)
        return cg_fail(ctx, CG_ERR_ARG, "cg_function_fill: unknown function kind %d", fn->kind);
    int mask = 0;
    for (int d = 0; d < f->ndim; ++d) mask |= (f->loc[d] & 1) << d;
    if ((rc = cg_check_field(ctx, grid, *f, f->dtype, mask, "f"))) return rc;
    if (f->dtype != CG_F32 && f->dtype != CG_F64) return cg_fail(ctx, CG_ERR_ARG, "cg_function_fill: bad dtype");
    cudaSetDevice(ctx->device);
    const int nd = grid->ndim;
    if (f->dtype == CG_F64)
        return nd == 1 ? fill_t<double, 1>(ctx, grid, fn, *f) : nd == 2 ? fill_t<double, 2>(ctx, grid, fn, *f)
                                                                        : fill_t<double, 3>(ctx, grid, fn, *f);
    return nd == 1 ? fill_t<float, 1>(ctx, grid, fn, *f) : nd == 2 ? fill_t<float, 2>(ctx, grid, fn, *f)
                                                                   : fill_t<float, 3>(ctx, grid, fn, *f);
}
