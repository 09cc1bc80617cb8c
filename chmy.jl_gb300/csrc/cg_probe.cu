// cg_probe.cu — the FP64 FMA throughput of the device, the roofline denominator of the kernels
// that are bound by the FP64 pipe rather than by HBM (GB300's FP64 rate is a small fraction of
// its FP32 rate).
#include "cg_common.cuh"

namespace {

constexpr int kChains = 8;  // independent FMA chains per thread: enough to fill the FP64 pipe

__global__ void __launch_bounds__(256) fp64_fma_kernel(double* out, int iters, double a, double b) {
    double x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-9;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int cg_fp64_peak(cg_ctx* ctx, double* flops) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_fp64_peak: ctx is NULL");
    if (!flops) return cg_fail(ctx, CG_ERR_ARG, "cg_fp64_peak: flops is NULL");
    cudaSetDevice(ctx->device);
    int bps = 0;
    CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fp64_fma_kernel, 256, 0));
    if (bps < 1) bps = 1;
    const int blocks = bps * ctx->num_sms, iters = 4096;
    double* sink = ctx->d_red ? reinterpret_cast<double*>(ctx->d_red) : nullptr;
    if (!sink) return cg_fail(ctx, CG_ERR_ARG, "cg_fp64_peak: context has no reduction scratch");
    fp64_fma_kernel<<<blocks, 256, 0, ctx->stream>>>(sink, iters, 0.999999, 1e-7);  // warm-up
    CG_CHECK_LAUNCH(ctx);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        CG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
        fp64_fma_kernel<<<blocks, 256, 0, ctx->stream>>>(sink, iters, 0.999999, 1e-7);
        CG_CHECK_LAUNCH(ctx);
        CG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
        CG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
        float ms = 0.f;
        CG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        best = ms < best ? ms : best;
    }
    *flops = 2.0 * kChains * (double)iters * blocks * 256 / (best * 1e-3);
    return CG_OK;
}
