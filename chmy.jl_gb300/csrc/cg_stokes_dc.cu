// cg_stokes_dc.cu — VE Stokes PT solve with FP32 pseudo-transient iterations inside an FP64
// defect-correction loop.
//
// Outer loop (FP64): the defect kernel evaluates the true residuals of the current FP64
// state — continuity R_P = divV, constitutive R_tau and momentum R_V — and the convergence
// measures of examples/stokes_2d_inc_ve_T.jl:154-157. The residuals are folded into the
// FP32 inputs of the UNCHANGED PT kernels: tau_old' = G dt R_tau (the constitutive residual
// of the correction then carries +R_tau), rho_g' = -R_V (the momentum residual carries
// +R_V) and a continuity forcing fP = R_P.
// Inner loop (FP32): PT iterations on the correction (dV, dP, dtau) from zero with
// homogeneous boundary conditions (same kinds, zero values), graph-replayed, until the
// FP32 measures fall below max(0.5 eps, inner_rtol * outer measure) or stagnate.
// Update (FP64): V += dV, P += dP, tau += dtau, then bc!(V).
#include "cg_march3d_tma.cuh"
#include "cg_stokes_kernels.cuh"

int cg_maxabs_enqueue(cg_ctx* ctx, int nfields, const cg_field* fields);
int cg_maxabs_collect(cg_ctx* ctx, int nfields, const cg_field* fields, double* out, int32_t* nonfinite);

namespace {
using namespace cgk;

struct DC32 {
    DF<float> fP, told[6], rho[3];
};

// FP64 residuals of the current state; FP32 forcing of the correction problem.
template <int ND>
__global__ void defect_kernel(const SV<double> v, const SP<double> s, const BodyFn<double> bf, const DC32 w, int e0,
                              int e1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    if (i > e0 || j > e1) return;
    const DF<double>& Vx = v.V[0];
    const DF<double>& Vy = v.V[1];
    const double exx = (Vx(i + 1, j, k) - Vx(i, j, k)) * s.idx[0];
    const double eyy = (Vy(i, j + 1, k) - Vy(i, j, k)) * s.idx[1];
    double dv = exx + eyy, ezz = 0.0;
    if (ND > 2) {
        ezz = (v.V[2](i, j, k + 1) - v.V[2](i, j, k)) * s.idx[2];
        dv = dv + ezz;
    }
    v.divV(i, j, k) = dv;
    w.fP(i, j, k) = (float)dv;
    const double Gdt = s.G * s.dt;
    double ieta_c = 0.0;
    if (v.has_eta) ieta_c = v.inv_eta(i, j, k);
    auto diag = [&](int c, double edd) {
        const double t = v.tau[c](i, j, k), to = v.tau_old[c](i, j, k);
        double r;
        if (v.has_eta)
            r = -(t - to) * s.inv_Gdt - t * ieta_c + 2.0 * (edd - dv * s.third);
        else
            r = -(t - to) / Gdt - t / s.eta + 2.0 * (edd - dv / 3.0);
        w.told[c](i, j, k) = (float)(Gdt * r);
    };
    auto shear = [&](int c, double eod, int a, int b) {
        const double t = v.tau[c](i, j, k), to = v.tau_old[c](i, j, k);
        double r;
        if (v.has_eta) {
            const int ai = a == 0, aj = a == 1, ak = a == 2;
            const int bi = b == 0, bj = b == 1, bk = b == 2;
            const double e00 = v.inv_eta(i - ai - bi, j - aj - bj, k - ak - bk);
            const double e10 = v.inv_eta(i - bi, j - bj, k - bk);
            const double e01 = v.inv_eta(i - ai, j - aj, k - ak);
            const double e11 = v.inv_eta(i, j, k);
            const double lo = fma(0.5, e10 - e00, e00);
            const double hi = fma(0.5, e11 - e01, e01);
            const double iev = fma(0.5, hi - lo, lo);
            r = -(t - to) * s.inv_Gdt - t * iev + 2.0 * eod;
        } else {
            r = -(t - to) / Gdt - t / s.eta + 2.0 * eod;
        }
        w.told[c](i, j, k) = (float)(Gdt * r);
    };
    const double exy = 0.5 * ((Vx(i, j, k) - Vx(i, j - 1, k)) * s.idx[1] + (Vy(i, j, k) - Vy(i - 1, j, k)) * s.idx[0]);
    if (ND == 2) {
        diag(0, exx);
        diag(1, eyy);
        shear(2, exy, 0, 1);
    } else {
        const DF<double>& Vz = v.V[2];
        const double exz = 0.5 * ((Vx(i, j, k) - Vx(i, j, k - 1)) * s.idx[2] + (Vz(i, j, k) - Vz(i - 1, j, k)) * s.idx[0]);
        const double eyz = 0.5 * ((Vy(i, j, k) - Vy(i, j, k - 1)) * s.idx[2] + (Vz(i, j, k) - Vz(i, j - 1, k)) * s.idx[1]);
        diag(0, exx);
        diag(1, eyy);
        diag(2, ezz);
        shear(3, exy, 0, 1);
        shear(4, exz, 0, 2);
        shear(5, eyz, 1, 2);
    }
    // momentum residuals at the faces of index I
    const DF<double>& P = v.P;
    const int XY = ND == 2 ? 2 : 3;
    const DF<double>& txx = v.tau[0];
    const DF<double>& tyy = v.tau[1];
    const DF<double>& txy = v.tau[XY];
    double rx = -((P(i, j, k) - P(i - 1, j, k)) * s.idx[0]) + (txx(i, j, k) - txx(i - 1, j, k)) * s.idx[0];
    rx = rx + (txy(i, j + 1, k) - txy(i, j, k)) * s.idx[1];
    double ry = -((P(i, j, k) - P(i, j - 1, k)) * s.idx[1]) + (tyy(i, j, k) - tyy(i, j - 1, k)) * s.idx[1];
    ry = ry + (txy(i + 1, j, k) - txy(i, j, k)) * s.idx[0];
    double rz = 0.0;
    if (ND > 2) {
        const DF<double>& tzz = v.tau[2];
        const DF<double>& txz = v.tau[4];
        const DF<double>& tyz = v.tau[5];
        rx = rx + (txz(i, j, k + 1) - txz(i, j, k)) * s.idx[2];
        ry = ry + (tyz(i, j, k + 1) - tyz(i, j, k)) * s.idx[2];
        rz = -((P(i, j, k) - P(i, j, k - 1)) * s.idx[2]) + (tzz(i, j, k) - tzz(i, j, k - 1)) * s.idx[2];
        rz = rz + (txz(i + 1, j, k) - txz(i, j, k)) * s.idx[0];
        rz = rz + (tyz(i, j + 1, k) - tyz(i, j, k)) * s.idx[1];
    }
    if (v.has_rho[0]) rx = rx - v.rho[0](i, j, k);
    else if (bf.fn[0].kind) rx = rx - body_fn(bf, 0, ND, i, j, k);
    if (v.has_rho[1]) ry = ry - v.rho[1](i, j, k);
    else if (bf.fn[1].kind) ry = ry - body_fn(bf, 1, ND, i, j, k);
    if (ND > 2 && v.has_rho[2]) rz = rz - v.rho[2](i, j, k);
    else if (ND > 2 && bf.fn[2].kind) rz = rz - body_fn(bf, 2, ND, i, j, k);
    v.rV[0](i, j, k) = rx;
    v.rV[1](i, j, k) = ry;
    w.rho[0](i, j, k) = (float)(-rx);
    w.rho[1](i, j, k) = (float)(-ry);
    if (ND > 2) {
        v.rV[2](i, j, k) = rz;
        w.rho[2](i, j, k) = (float)(-rz);
    }
}

// dst += src over whole padded arrays (logical -1 .. n+2 with H = 1), one launch for a table.
constexpr int kMaxUpd = 10;
struct UpdItem {
    DF<double> dst;
    DF<float> src;
    int n0, n1, n2;  // padded extents (n + 4)
};
struct UpdTable {
    int count;
    UpdItem it[kMaxUpd];
};

__global__ void update_kernel(const UpdTable t) {
    const UpdItem u = t.it[blockIdx.y];
    const long plane = (long)u.n0 * u.n1;
    const long total = plane * u.n2;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int k = (int)(q / plane);
        const long r = q - (long)k * plane;
        const int j = (int)(r / u.n0);
        const int i = (int)(r - (long)j * u.n0);
        // logical index = padded index - 1 in every used dim
        const int li = i - 1, lj = u.n1 > 1 ? j - 1 : 0, lk = u.n2 > 1 ? k - 1 : 0;
        double* d = u.dst.ptr(li, lj, lk);
        *d = *d + (double)u.src(li, lj, lk);
    }
}

struct Work {
    cg_field dV[3], dP, dtau[6], told[6], fP, rho[3], ieta, divV, rV[3];
    cg_field dV2[3], dP2, dtau2[6];  // ping-pong partners of the fused 2D kernel
};

// FP32 field like `f` (same extents, locations, halo 1) with x rows of `pitch` elements and, in
// 3D, planes of `rows` rows. All work arrays share the row and plane strides, so the fused
// kernels address every array with one offset.
cg_field like32(const cg_field& f, long pitch, long rows, long front, char*& cursor, size_t& bytes, bool dry) {
    cg_field g;
    std::memset(&g, 0, sizeof(g));
    g.dtype = CG_F32;
    g.ndim = f.ndim;
    long ext[3] = {1, 1, 1};
    for (int d = 0; d < 3; ++d) {
        g.n[d] = f.n[d];
        g.loc[d] = f.loc[d];
        g.halo[d] = d < f.ndim ? 1 : 0;
        if (d < f.ndim) ext[d] = f.n[d] + 4;
    }
    if (f.ndim > 1) ext[0] = pitch;
    if (f.ndim > 2) ext[1] = rows;
    g.stride[0] = 1;
    g.stride[1] = f.ndim > 1 ? ext[0] : 0;
    g.stride[2] = f.ndim > 2 ? ext[0] * ext[1] : 0;
    const size_t sz = (((size_t)ext[0] * ext[1] * ext[2] + (size_t)front) * 4 + 255) & ~(size_t)255;
    if (!dry) g.data = cursor + front * 4;
    cursor += sz;
    bytes += sz;
    return g;
}

int make_work(cg_ctx* ctx, const cg_stokes_fields* f, int nd, Work* w) {
    const int nt = nd == 2 ? 3 : 6;
    // 3D: every array's data pointer sits `front` elements past a 256-byte boundary, so that
    // logical x index 0 of every row starts a 128-byte line (measured 2 % faster for the 3D
    // kernel than rows whose first padded element starts a line); 2D: the first padded element
    const long front = nd == 3 ? 31 : 0;
    // the widest x extent (V.x is Vertex in x) after the front offset, rounded up to 32
    // elements (128 bytes)
    const long pitch = (front + (long)f->V[0].n[0] + 4 + 31) / 32 * 32;
    // the widest y extent (V.y is Vertex in y): rows per plane in 3D
    const long rows = (long)f->V[1].n[1] + 4;
    for (int pass = 0; pass < 2; ++pass) {
        const bool dry = pass == 0;
        char* cur = dry ? nullptr : static_cast<char*>(ctx->dc_pool);
        size_t bytes = 0;
        for (int d = 0; d < nd; ++d) {
            w->dV[d] = like32(f->V[d], pitch, rows, front, cur, bytes, dry);
            w->dV2[d] = like32(f->V[d], pitch, rows, front, cur, bytes, dry);
            w->rho[d] = like32(f->V[d], pitch, rows, front, cur, bytes, dry);
            w->rV[d] = like32(f->V[d], pitch, rows, front, cur, bytes, dry);
        }
        w->dP = like32(f->P, pitch, rows, front, cur, bytes, dry);
        w->dP2 = like32(f->P, pitch, rows, front, cur, bytes, dry);
        w->fP = like32(f->P, pitch, rows, front, cur, bytes, dry);
        w->ieta = like32(f->P, pitch, rows, front, cur, bytes, dry);
        w->divV = like32(f->P, pitch, rows, front, cur, bytes, dry);
        for (int c = 0; c < nt; ++c) {
            w->dtau[c] = like32(f->tau[c], pitch, rows, front, cur, bytes, dry);
            w->dtau2[c] = like32(f->tau[c], pitch, rows, front, cur, bytes, dry);
            w->told[c] = like32(f->tau[c], pitch, rows, front, cur, bytes, dry);
        }
        if (dry && bytes > ctx->dc_pool_bytes) {
            if (ctx->dc_pool) {
                CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                CG_CUDA(ctx, cudaFree(ctx->dc_pool));
                ctx->dc_pool = nullptr;
                ctx->dc_pool_bytes = 0;
            }
            CG_CUDA(ctx, cudaMalloc(&ctx->dc_pool, bytes));
            CG_CUDA(ctx, cudaMemsetAsync(ctx->dc_pool, 0, bytes, ctx->stream));
            ctx->dc_pool_bytes = bytes;
        }
    }
    return CG_OK;
}

// Elements spanned by a work array (halo 1, rows of stride[1] elements).
size_t padded_count(const cg_field& f) {
    if (f.ndim == 1) return (size_t)f.n[0] + 4;
    if (f.ndim == 2) return (size_t)f.stride[1] * (f.n[1] + 4);
    return (size_t)f.stride[2] * (f.n[2] + 4);
}

// max |r_tau| of the FP32 correction over the interior of every stress component: the inner
// loop's constitutive measure, the FP32 counterpart of the outer err_tau. Without it, a state
// whose momentum and continuity residuals vanish (a uniform stress correction) would end the
// inner loop at its first check. The maximum is kept as the bits of |r| (a NaN's bits exceed
// every finite value's, so a non-finite residual is reported).
template <int ND>
__global__ void tau_res_kernel(const SV<float> v, const SP<float> s, int e0, int e1, int n0, int n1, int n2,
                               unsigned long long* slot) {
    // one thread per point of the launch range; the block's maximum goes into the slot, with an
    // atomic only when it exceeds the slot's current value (one address: atomics from every warp
    // of the grid would serialise there)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ND > 2 ? blockIdx.z : 0;
    unsigned m = 0;
    {
        if (i <= e0 && j <= e1) {
            // interior test per location: logical index 1..n (Center) or 1..n+1 (Vertex) along
            // each dim (0 is the lower ghost layer of the launch range)
            auto in = [&](int li, int lj, int lk) {
                return i >= 1 && j >= 1 && i <= n0 + li && j <= n1 + lj && (ND < 3 || (k >= 1 && k <= n2 + lk));
            };
            auto take = [&](float r) { m = max(m, __float_as_uint(fabsf(r))); };
            const float exx = (v.V[0](i + 1, j, k) - v.V[0](i, j, k)) * s.idx[0];
            const float eyy = (v.V[1](i, j + 1, k) - v.V[1](i, j, k)) * s.idx[1];
            float ezz = 0.f, dv = exx + eyy;
            if (ND > 2) {
                ezz = (v.V[2](i, j, k + 1) - v.V[2](i, j, k)) * s.idx[2];
                dv = dv + ezz;
            }
            const float ie = v.ieta(i, j, k);
            auto diag = [&](int c, float e) {
                const float t = v.tau[c](i, j, k);
                take(-(t - v.tau_old[c](i, j, k)) * s.inv_Gdt - t * ie + 2.f * (e - dv * s.third));
            };
            auto shear = [&](int c, float e, int a, int b) {
                const float t = v.tau[c](i, j, k);
                const float iev = shear_inv_eta(v, i, j, k, a, b);
                take(-(t - v.tau_old[c](i, j, k)) * s.inv_Gdt - t * iev + 2.f * e);
            };
            const float exy = 0.5f * ((v.V[0](i, j, k) - v.V[0](i, j - 1, k)) * s.idx[1] +
                                      (v.V[1](i, j, k) - v.V[1](i - 1, j, k)) * s.idx[0]);
            if (in(0, 0, 0)) {
                diag(0, exx);
                diag(1, eyy);
                if (ND > 2) diag(2, ezz);
            }
            if (ND == 2) {
                if (in(1, 1, 0)) shear(2, exy, 0, 1);
            } else {
                const float exz = 0.5f * ((v.V[0](i, j, k) - v.V[0](i, j, k - 1)) * s.idx[2] +
                                          (v.V[2](i, j, k) - v.V[2](i - 1, j, k)) * s.idx[0]);
                const float eyz = 0.5f * ((v.V[1](i, j, k) - v.V[1](i, j, k - 1)) * s.idx[2] +
                                          (v.V[2](i, j, k) - v.V[2](i, j - 1, k)) * s.idx[1]);
                if (in(1, 1, 0)) shear(3, exy, 0, 1);
                if (in(1, 0, 1)) shear(4, exz, 0, 2);
                if (in(0, 1, 1)) shear(5, eyz, 1, 2);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ unsigned sm[32];
    const int t = threadIdx.y * blockDim.x + threadIdx.x, lane = t & 31, w = t >> 5;
    if (lane == 0) sm[w] = m;
    __syncthreads();
    if (w == 0) {
        const int nwarp = (int)(blockDim.x * blockDim.y) >> 5;
        m = lane < nwarp ? sm[lane] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0 && m && (unsigned long long)m > *reinterpret_cast<volatile unsigned long long*>(slot))
            atomicMax(slot, (unsigned long long)m);
    }
}

__global__ void fill_kernel(float* dst, float v, size_t count) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (size_t)gridDim.x * blockDim.x)
        dst[q] = v;
}

__global__ void reciprocal_kernel(float* dst, const double* src, long dst_s1, long dst_s2, long src_s1, long src_s2,
                                  int n0, int n1, int n2) {
    const long plane = (long)n0 * n1;
    const long total = plane * n2;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int k = (int)(q / plane);
        const long r = q - (long)k * plane;
        const int j = (int)(r / n0);
        const int i = (int)(r - (long)j * n0);
        dst[i + j * dst_s1 + k * dst_s2] = (float)(1.0 / src[i + j * src_s1 + k * src_s2]);
    }
}

}  // namespace

int cg_stokes_solve_dc(cg_ctx* ctx, const cg_grid* g, const cg_stokes_fields* f, const cg_stokes_params* p,
                       const cg_bc* bc_V, const cg_solve_opts* o, cg_solve_result* res) {
    const int nd = g->ndim;
    const int nt = nd == 2 ? 3 : 6;
    for (int d = 0; d < nd; ++d)
        if (f->V[d].halo[d] != 1) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve (FP32): halo 1 fields only");
    for (int c = 0; c < nt; ++c)
        if (f->tau[c].halo[0] != 1) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve (FP32): halo 1 fields only");
    if (f->P.halo[0] != 1) return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve (FP32): halo 1 fields only");
    Work w;
    int rc = make_work(ctx, f, nd, &w);
    if (rc) return rc;
    std::memset(res, 0, sizeof(*res));
    CG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));

    // FP32 1/eta (and its use flag) for the correction operator
    const bool var = cg_present(f->eta) || cg_present(f->inv_eta);
    if (var) {
        const cg_field& e = cg_present(f->eta) ? f->eta : f->inv_eta;
        const int n0 = e.n[0] + 4, n1 = nd > 1 ? e.n[1] + 4 : 1, n2 = nd > 2 ? e.n[2] + 4 : 1;
        if (cg_present(f->eta)) {
            reciprocal_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(
                static_cast<float*>(w.ieta.data), static_cast<const double*>(e.data), w.ieta.stride[1], w.ieta.stride[2],
                e.stride[1], e.stride[2], n0, n1, n2);
        } else {
            return cg_fail(ctx, CG_ERR_UNSUPPORTED, "stokes_solve (FP32): pass eta (inv_eta alone is not enough)");
        }
        CG_CHECK_LAUNCH(ctx);
    } else {
        // scalar viscosity: the fused kernels take 1/eta per cell, here a constant
        fill_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(static_cast<float*>(w.ieta.data),
                                                               (float)(1.0 / p->eta), padded_count(w.ieta));
        CG_CHECK_LAUNCH(ctx);
    }

    // FP64 views of the state and FP32 views of the correction
    SV<double> v64 = views<double>(f, nd);
    v64.has_rV = 1;
    v64.has_divV = 1;
    const SP<double> s64 = scalars<double>(g, p);
    const BodyFn<double> bf64 = body_fns<double>(g, p);
    DC32 d32;
    std::memset(&d32, 0, sizeof(d32));
    d32.fP = cg_view<float>(w.fP);
    for (int c = 0; c < nt; ++c) d32.told[c] = cg_view<float>(w.told[c]);
    for (int d = 0; d < nd; ++d) d32.rho[d] = cg_view<float>(w.rho[d]);

    cg_stokes_fields f32;
    std::memset(&f32, 0, sizeof(f32));
    for (int d = 0; d < nd; ++d) {
        f32.V[d] = w.dV[d];
        f32.r_V[d] = w.rV[d];
        f32.rho_g[d] = w.rho[d];
    }
    f32.P = w.dP;
    f32.divV = w.divV;
    for (int c = 0; c < nt; ++c) {
        f32.tau[c] = w.dtau[c];
        f32.tau_old[c] = w.told[c];
    }
    f32.inv_eta = w.ieta;
    const SV<float> v32 = views<float>(&f32, nd);
    const SP<float> s32 = scalars<float>(g, p);

    cg_bc bc0[3];
    for (int d = 0; d < nd; ++d) {
        bc0[d] = bc_V ? bc_V[d] : cg_bc{};
        for (int a = 0; a < 3; ++a) {
            bc0[d].value[a][0] = bc0[d].value[a][1] = 0.0;
            bc0[d].values[a][0] = bc0[d].values[a][1] = nullptr;
        }
    }
    // FP64 measures: divV, r_V (the reference's) and the constitutive residuals, read from the
    // FP32 forcing tau_old' = G dt R_tau (the initial guess of a PT solve can have zero divV and
    // r_V while tau is far from its constitutive value)
    cg_field red64[4 + 6], red32[5];
    red64[0] = f->divV;
    red32[0] = w.divV;
    for (int d = 0; d < nd; ++d) {
        red64[1 + d] = f->r_V[d];
        red32[1 + d] = w.rV[d];
    }
    for (int c = 0; c < nt; ++c) red64[1 + nd + c] = w.told[c];
    red32[nd + 1] = w.told[0];  // FP32 slot of the constitutive measure (only its dtype is read)
    cg_bc rbc[3];
    std::memset(rbc, 0, sizeof(rbc));
    for (int d = 0; d < nd; ++d) rbc[d].kind[d][0] = rbc[d].kind[d][1] = CG_BC_DIRICHLET;

    UpdTable upd;
    std::memset(&upd, 0, sizeof(upd));
    auto add_upd = [&](const cg_field& dst, const cg_field& src) {
        UpdItem& u = upd.it[upd.count++];
        u.dst = cg_view<double>(dst);
        u.src = cg_view<float>(src);
        u.n0 = dst.n[0] + 4;
        u.n1 = nd > 1 ? dst.n[1] + 4 : 1;
        u.n2 = nd > 2 ? dst.n[2] + 4 : 1;
    };
    for (int d = 0; d < nd; ++d) add_upd(f->V[d], w.dV[d]);
    add_upd(f->P, w.dP);
    for (int c = 0; c < nt; ++c) add_upd(f->tau[c], w.dtau[c]);

    const dim3 block(32, 8);
    const dim3 grid3(cg_div_up(g->n[0] + 2, block.x), cg_div_up(g->n[1] + 2, block.y), nd > 2 ? g->n[2] + 2 : 1);
    const int e0 = g->n[0] + 1, e1 = g->n[1] + 1;
    const int ncheck = o->ncheck;
    const double inner_rtol = o->inner_rtol > 0 ? o->inner_rtol : 1e-5;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 8;
    int total_iter = 0, status = CG_ERR_NOCONV;

    // the PT chunk of the correction, captured once and replayed
    std::string key = "stokes_dc_chunk";
    cg_key_add(key, *g);
    cg_key_add(key, f32);
    cg_key_add(key, *p);
    cg_key_add(key, ncheck);
    // 2D: fused kernel, ping-pong A -> B -> A, an even number of iterations per chunk
    Fused2D<float> fa, fb;
    std::memset(&fa, 0, sizeof(fa));
    if (nd == 2) {
        fa.txx_o = cg_view<float>(w.told[0]);
        fa.tyy_o = cg_view<float>(w.told[1]);
        fa.txy_o = cg_view<float>(w.told[2]);
        fa.ieta = cg_view<float>(w.ieta);
        fa.fP = cg_view<float>(w.fP);
        fa.has_fP = 1;
        fa.rhox = cg_view<float>(w.rho[0]);
        fa.rhoy = cg_view<float>(w.rho[1]);
        fa.has_rho = 1;
        fa.divV = cg_view<float>(w.divV);
        fa.rVx = cg_view<float>(w.rV[0]);
        fa.rVy = cg_view<float>(w.rV[1]);
        fb = fa;
        fa.Vx_in = fb.Vx_out = cg_view<float>(w.dV[0]);
        fa.Vy_in = fb.Vy_out = cg_view<float>(w.dV[1]);
        fa.txx_in = fb.txx_out = cg_view<float>(w.dtau[0]);
        fa.tyy_in = fb.tyy_out = cg_view<float>(w.dtau[1]);
        fa.txy_in = fb.txy_out = cg_view<float>(w.dtau[2]);
        fa.P_in = fb.P_out = cg_view<float>(w.dP);
        fa.Vx_out = fb.Vx_in = cg_view<float>(w.dV2[0]);
        fa.Vy_out = fb.Vy_in = cg_view<float>(w.dV2[1]);
        fa.txx_out = fb.txx_in = cg_view<float>(w.dtau2[0]);
        fa.tyy_out = fb.tyy_in = cg_view<float>(w.dtau2[1]);
        fa.txy_out = fb.txy_in = cg_view<float>(w.dtau2[2]);
        fa.P_out = fb.P_in = cg_view<float>(w.dP2);
    }
    // 3D: the z-marching fused kernel, ping-pong the same way
    Fused3D<float> ga, gb;
    std::memset(&ga, 0, sizeof(ga));
    if (nd == 3) {
        for (int c = 0; c < 6; ++c) ga.tau_o[c] = cg_view<float>(w.told[c]);
        ga.ieta = cg_view<float>(w.ieta);
        ga.fP = cg_view<float>(w.fP);
        ga.has_fP = 1;
        for (int d = 0; d < 3; ++d) {
            ga.rho[d] = cg_view<float>(w.rho[d]);
            ga.has_rho[d] = 1;
            ga.rV[d] = cg_view<float>(w.rV[d]);
        }
        ga.divV = cg_view<float>(w.divV);
        gb = ga;
        for (int d = 0; d < 3; ++d) {
            ga.V_in[d] = gb.V_out[d] = cg_view<float>(w.dV[d]);
            ga.V_out[d] = gb.V_in[d] = cg_view<float>(w.dV2[d]);
        }
        for (int c = 0; c < 6; ++c) {
            ga.tau_in[c] = gb.tau_out[c] = cg_view<float>(w.dtau[c]);
            ga.tau_out[c] = gb.tau_in[c] = cg_view<float>(w.dtau2[c]);
        }
        ga.P_in = gb.P_out = cg_view<float>(w.dP);
        ga.P_out = gb.P_in = cg_view<float>(w.dP2);
    }
    // tensor maps of the TMA-fed 3D variants (A -> B reads dV, dP, dtau; B -> A the partners)
    m3t::Tma tma;
    int* terr = nullptr;
    if (nd == 3) {
        terr = cg_tma_flag(ctx, &rc);
        if (rc) return rc;
        const cg_field* Va[3] = {&w.dV[0], &w.dV[1], &w.dV[2]};
        const cg_field* Vb[3] = {&w.dV2[0], &w.dV2[1], &w.dV2[2]};
        const cg_field *ta[6], *tb[6], *to[6];
        for (int c = 0; c < 6; ++c) {
            ta[c] = &w.dtau[c];
            tb[c] = &w.dtau2[c];
            to[c] = &w.told[c];
        }
        const cg_field* rho[3] = {&w.rho[0], &w.rho[1], &w.rho[2]};
        tma = m3t::make_tma(Va, &w.dP, ta, Vb, &w.dP2, tb, &w.ieta, to, &w.fP, rho, g->n, terr);
    }
    const M3Launch lga = m3_launch_of(&tma, true), lgb = m3_launch_of(&tma, false);
    const int nchunk = ncheck + (ncheck & 1);
    cg_key_add(key, nchunk);
    // 2D: bc!(dV) folded into the velocity reads from the chunk's second iteration on; the
    // chunk's last output (dV: nchunk is even) is patched once at its end
    const Fused2D<float> fa0 = fa;
    VFold<float> vf;
    const bool fold = nd == 2 && cg_bc_fold_enabled() && make_vfold(g, bc0, &vf);
    if (fold) fa.bc = fb.bc = vf;
    cg_key_add(key, (int)fold);
    // launch layout of the fused kernel, timed on the work buffers (A -> B) before capture
    const cg_tune_cfg tc = nd == 2 ? tune_march2d(fa, s32, g->n[0], g->n[1], ctx->num_sms, ctx->stream)
                                   : tune_march3d(ga, s32, g->n[0], g->n[1], g->n[2], ctx->num_sms, ctx->stream, lga);
    cg_key_add(key, tc);
    const bool staged = nd == 3 && tma.ok && tc.variant >= kM3TmaFirst;
    if (staged) cg_key_add(key, cg_tma_wait_cfg());
    // two iterations per pass (the tuner's variant 1) where bc!(dV) is folded into the reads:
    // passes alternate A -> B and B -> A, and an odd count of passes leaves its last two
    // iterations to the one-iteration kernel, so that the chunk ends in A
    const bool x2 = nd == 2 && fold && tc.variant >= 1;
    const int npass = x2 ? (nchunk / 2) - ((nchunk / 2) & 1) : 0;
    auto chunk = [&]() {
        return cg_graph_run(ctx, key, [&](cudaStream_t st) {
            for (int k = 0; k < npass; ++k) {
                const bool last = 2 * k + 2 == nchunk;
                const Fused2D<float>& fk = (k % 2 == 0) ? fa : fb;
                const int nsm = ctx->num_sms;
                const cudaError_t le =
                    last ? launch_march2d_x2<float, true>(fk, s32, g->n[0], g->n[1], nsm, tc.seg, k > 0, st, k > 0, tc.variant)
                         : launch_march2d_x2<float, false>(fk, s32, g->n[0], g->n[1], nsm, tc.seg, k > 0, st, k > 0, tc.variant);
                if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused2d x2 launch: %s", cudaGetErrorString(le));
                if (last) {
                    int r = cg_bc_apply_impl(ctx, g, nd, w.dV, bc0, true);
                    if (r) return r;
                }
            }
            for (int it = 2 * npass; it < nchunk; ++it) {
                const bool last = it == nchunk - 1;
                if (nd == 2) {
                    const Fused2D<float>& fk = it == 0 ? fa0 : (it % 2 == 0) ? fa : fb;
                    const int nsm = ctx->num_sms;
                    const cudaError_t le = last ? launch_march2d<float, true>(fk, s32, g->n[0], g->n[1], nsm, tc.seg, st, it > 0)
                                                : launch_march2d<float, false>(fk, s32, g->n[0], g->n[1], nsm, tc.seg, st, it > 0);
                    if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused2d launch: %s", cudaGetErrorString(le));
                    if (!fold || last) {
                        int r = cg_bc_apply_impl(ctx, g, nd, (it % 2 == 0) ? w.dV2 : w.dV, bc0, true);
                        if (r) return r;
                    }
                } else {
                    const Fused3D<float>& fk = (it % 2 == 0) ? ga : gb;
                    const M3Launch& lk = (it % 2 == 0) ? lga : lgb;
                    const int nsm = ctx->num_sms;
                    const cudaError_t le =
                        last ? launch_march3d_any<float, true>(fk, s32, g->n[0], g->n[1], g->n[2], nsm, tc.seg, st, tc.variant,
                                                               it > 0, lk)
                             : launch_march3d_any<float, false>(fk, s32, g->n[0], g->n[1], g->n[2], nsm, tc.seg, st,
                                                                tc.variant, it > 0, lk);
                    if (le != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "fused3d launch: %s", cudaGetErrorString(le));
                    // no dependent launches around the TMA-fed kernel (measured slower with them)
                    int r = cg_bc_apply_impl(ctx, g, nd, (it % 2 == 0) ? w.dV2 : w.dV, bc0, !staged);
                    if (r) return r;
                }
            }
            return (int)CG_OK;
        });
    };

    double outer_err[4] = {0, 0, 0, 0};
    for (int outer = 0; outer <= max_outer; ++outer) {
        // FP64 defect of the current state
        if (nd == 2) defect_kernel<2><<<grid3, block, 0, ctx->stream>>>(v64, s64, bf64, d32, e0, e1);
        else defect_kernel<3><<<grid3, block, 0, ctx->stream>>>(v64, s64, bf64, d32, e0, e1);
        CG_CHECK_LAUNCH(ctx);
        if ((rc = cg_bc_apply_impl(ctx, g, nd, f->r_V, rbc))) return rc;
        if ((rc = cg_maxabs_enqueue(ctx, nd + 1 + nt, red64))) return rc;
        double m[4 + 6];
        int32_t bad = 0;
        if ((rc = cg_maxabs_collect(ctx, nd + 1 + nt, red64, m, &bad))) return rc;
        res->checks++;
        outer_err[0] = m[0] * o->tau_scale;
        for (int d = 0; d < nd; ++d) outer_err[1 + d] = m[1 + d] * o->v_scale;
        for (int c = 0; c <= nd; ++c) res->err[c] = outer_err[c];
        double etau = 0.0;
        for (int c = 0; c < nt; ++c) etau = std::max(etau, m[1 + nd + c]);
        res->err_tau = etau / (p->G * p->dt) * o->tau_scale;
        if (bad) {
            status = CG_ERR_NONFINITE;
            cg_fail(ctx, CG_ERR_NONFINITE, "stokes_solve (FP32): non-finite FP64 residual");
            break;
        }
        double emax = res->err_tau;
        for (int c = 0; c <= nd; ++c) emax = std::max(emax, outer_err[c]);
        if (emax < o->eps) {
            status = CG_OK;
            res->converged = 1;
            break;
        }
        if (outer == max_outer || total_iter >= o->max_iter) break;
        // FP32 correction solve from zero
        for (int d = 0; d < nd; ++d) {
            CG_CUDA(ctx, cudaMemsetAsync(w.dV[d].data, 0, padded_count(w.dV[d]) * 4, ctx->stream));
            CG_CUDA(ctx, cudaMemsetAsync(w.dV2[d].data, 0, padded_count(w.dV2[d]) * 4, ctx->stream));
        }
        CG_CUDA(ctx, cudaMemsetAsync(w.dP.data, 0, padded_count(w.dP) * 4, ctx->stream));
        CG_CUDA(ctx, cudaMemsetAsync(w.dP2.data, 0, padded_count(w.dP2) * 4, ctx->stream));
        for (int c = 0; c < nt; ++c) {
            CG_CUDA(ctx, cudaMemsetAsync(w.dtau[c].data, 0, padded_count(w.dtau[c]) * 4, ctx->stream));
            CG_CUDA(ctx, cudaMemsetAsync(w.dtau2[c].data, 0, padded_count(w.dtau2[c]) * 4, ctx->stream));
        }
        const double target = std::max(0.5 * o->eps, inner_rtol * emax);
        // stagnation: no 10% gain over a window of 4 n iterations (accelerated PT converges
        // with oscillations of that period, so shorter windows stop it too early)
        const int nmax = std::max(g->n[0], std::max(g->n[1], nd > 2 ? g->n[2] : 1));
        const int window = std::max(4 * nchunk, 4 * nmax);
        double best = 1e300;
        int since_best = 0;
        while (total_iter < o->max_iter) {
            if ((rc = chunk())) return rc;
            if (staged && (rc = cg_tma_check(ctx, terr, "fused3d iteration"))) return rc;
            total_iter += nchunk;
            if ((rc = cg_bc_apply_impl(ctx, g, nd, f32.r_V, rbc))) return rc;
            if ((rc = cg_maxabs_enqueue(ctx, nd + 1, red32))) return rc;
            // the constitutive measure into the next reduction slot
            CG_CUDA(ctx, cudaMemsetAsync(ctx->d_red + nd + 1, 0, sizeof(unsigned long long), ctx->stream));
            if (nd == 2)
                tau_res_kernel<2><<<grid3, block, 0, ctx->stream>>>(v32, s32, e0, e1, g->n[0], g->n[1], 1,
                                                                     ctx->d_red + nd + 1);
            else
                tau_res_kernel<3><<<grid3, block, 0, ctx->stream>>>(v32, s32, e0, e1, g->n[0], g->n[1], g->n[2],
                                                                     ctx->d_red + nd + 1);
            CG_CHECK_LAUNCH(ctx);
            double e32[5];
            if ((rc = cg_maxabs_collect(ctx, nd + 2, red32, e32, &bad))) return rc;
            res->checks++;
            if (bad) {
                status = CG_ERR_NONFINITE;
                cg_fail(ctx, CG_ERR_NONFINITE, "stokes_solve (FP32): non-finite correction residual");
                break;
            }
            double em = std::max(e32[0], e32[nd + 1]) * o->tau_scale;
            for (int d = 0; d < nd; ++d) em = std::max(em, e32[1 + d] * o->v_scale);
            if (em < target) break;
            if (em < 0.9 * best) {
                best = em;
                since_best = 0;
            } else if ((since_best += nchunk) >= window) {
                break;  // FP32 floor reached: hand back to the FP64 defect
            }
        }
        if (status == CG_ERR_NONFINITE) break;
        // FP64 update and boundary values
        update_kernel<<<dim3(ctx->num_sms * 2, upd.count), 256, 0, ctx->stream>>>(upd);
        CG_CHECK_LAUNCH(ctx);
        if ((rc = cg_bc_apply_impl(ctx, g, nd, f->V, bc_V))) return rc;
        res->outer++;
    }
    CG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    CG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    res->seconds = ms * 1e-3;
    res->iterations = total_iter;
    if (status == CG_ERR_NOCONV)
        cg_fail(ctx, CG_ERR_NOCONV, "stokes_solve (FP32): not converged after %d iterations, %d corrections",
                total_iter, res->outer);
    return status;
}
