// qew_peak.cu -- the FP64 roof of this GPU, measured.
//
// The plain FP64 gather is bound by the FP64 pipe, not by HBM, so its
// roofline needs the FP64 instruction rate of the part: a grid of eight
// resident CTAs per SM, each thread running eight independent FMA chains
// (enough independent work to keep the pipe full), timed with CUDA events on
// the context's stream. No reference counterpart (a measurement helper of
// the benchmark).
#include "qew_internal.cuh"

namespace {

constexpr int kPeakBS = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kPeakBS)
k_fp64_fma_rate(int iters, double b, double c, double *sink) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = (double)(threadIdx.x + k) * 1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == 12345.678) *sink = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" qew_status qew_measure_fp64_fma_rate(qew_ctx *ctx, int iters, double *fma_per_s,
                                                double *ms_out) {
    if (!ctx || !fma_per_s || iters < 1 || iters > (1 << 24))
        return qew_fail(ctx, QEW_ERR_INVALID, "measure_fp64_fma_rate: bad arguments");
    QEW_TRY(qew_scratch_reserve(ctx, 256));
    const int blocks = ctx->num_sms * 8;
    cudaEvent_t e0, e1;
    QEW_CUDA(ctx, cudaEventCreate(&e0));
    QEW_CUDA(ctx, cudaEventCreate(&e1));
    double *sink = (double *)ctx->scratch;
    // one untimed launch, then the timed one
    k_fp64_fma_rate<<<blocks, kPeakBS, 0, ctx->stream>>>(iters / 8 + 1, 0.999999, 1e-7, sink);
    cudaEventRecord(e0, ctx->stream);
    k_fp64_fma_rate<<<blocks, kPeakBS, 0, ctx->stream>>>(iters, 0.999999, 1e-7, sink);
    cudaEventRecord(e1, ctx->stream);
    const qew_status st = qew_launch_check(ctx, "fp64_fma_rate", 2);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != QEW_OK) return st;
    if (e != cudaSuccess)
        return qew_fail(ctx, QEW_ERR_CUDA, "measure_fp64_fma_rate: %s", cudaGetErrorString(e));
    const double fmas = (double)blocks * kPeakBS * kChains * (double)iters;
    *fma_per_s = fmas / (ms * 1e-3);
    if (ms_out) *ms_out = ms;
    return QEW_OK;
}
