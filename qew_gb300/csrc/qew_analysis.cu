// qew_analysis.cu -- roughness statistics of relaxed lines on the device: the
// height-difference autocorrelation and the power spectrum that the
// reference's post-processing adds beside every profile (ell, acf, q, psd;
// tools/postprocess_static.py:38-46). The reference computes them with an
// external package that is not part of its tree, so the definitions are
// stated here (and in include/qew_gpu.h) and tested against direct sums:
//   dx = L / n,  H_k = sum_i h_i exp(-2 pi i i k / n)  (k = 0 .. n/2)
//   ell_k = k dx,  acf_k = (1/n) sum_i (h_{(i+k) mod n} - h_i)^2
//   q_k = 2 pi k / L,  psd_k = (dx / n) |H_k|^2
// acf comes from the spectrum (Wiener-Khinchin): with
// R_k = (1/n) sum_i h_i h_{i+k} = IFFT(|H|^2)_k / n, acf_k = 2 (R_0 - R_k).
// Lines of one batch are n apart; cuFFT does the transforms for all of them.
#include <cufft.h>

#include "qew_internal.cuh"

namespace {

constexpr int kBS = 256;

// |H_k|^2 -> psd (dx / n scale) and the real spectrum for the inverse
// transform (in place in `spec`).
__global__ void k_power(cufftDoubleComplex *__restrict__ spec, long total, int nh, int n, double L,
                        double *__restrict__ q, double *__restrict__ psd) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int k = (int)(t % nh);
    const cufftDoubleComplex c = spec[t];
    const double p2 = c.x * c.x + c.y * c.y;
    const double dx = L / (double)n;
    if (psd) psd[t] = dx / (double)n * p2;
    if (q && t < nh) q[k] = 2.0 * 3.14159265358979323846 * (double)k / L;
    spec[t] = cufftDoubleComplex{p2, 0.0};
}

// acf_k = 2 (R_0 - R_k), R = IFFT(|H|^2) / n (cuFFT's inverse is unscaled:
// divide by n twice, once for the inverse transform and once for the mean).
__global__ void k_acf(const double *__restrict__ r, long lines, int n, int nh, double L,
                      double *__restrict__ ell, double *__restrict__ acf) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= lines * nh) return;
    const long line = t / nh;
    const int k = (int)(t % nh);
    const double inv = 1.0 / ((double)n * (double)n);
    const double *rl = r + line * n;
    acf[t] = 2.0 * (rl[0] - rl[k]) * inv;
    if (ell && t < nh) ell[k] = (double)k * (L / (double)n);
}

}  // namespace

extern "C" qew_status qew_line_statistics(qew_ctx *ctx, int count, const double *d_h, int n,
                                          double physical_size, double *d_ell, double *d_acf,
                                          double *d_q, double *d_psd) {
    QEW_RANGE();
    if (!ctx || count < 1 || !d_h || n < 2 || !(physical_size > 0) || (!d_acf && !d_psd))
        return qew_fail(ctx, QEW_ERR_INVALID, "line_statistics: bad arguments");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nh = n / 2 + 1;
    const size_t spec_b = (size_t)count * nh * sizeof(cufftDoubleComplex);
    const size_t r_off = (spec_b + 255) & ~size_t(255);
    QEW_TRY(qew_scratch_reserve(ctx, r_off + (size_t)count * n * sizeof(double) + 256));
    cufftDoubleComplex *spec = (cufftDoubleComplex *)ctx->scratch;
    double *r = (double *)((char *)ctx->scratch + r_off);
    cufftHandle fwd = 0, inv = 0;
    bool have_fwd = false, have_inv = false;
    auto done = [&](qew_status st) {
        if (have_fwd || have_inv) cudaStreamSynchronize(ctx->stream);
        if (have_fwd) cufftDestroy(fwd);
        if (have_inv) cufftDestroy(inv);
        return st;
    };
    int dims[1] = {n};
    if (cufftPlanMany(&fwd, 1, dims, nullptr, 1, n, nullptr, 1, nh, CUFFT_D2Z, count) != CUFFT_SUCCESS)
        return done(qew_fail(ctx, QEW_ERR_CUDA, "line_statistics: cuFFT plan"));
    have_fwd = true;
    if (cufftPlanMany(&inv, 1, dims, nullptr, 1, nh, nullptr, 1, n, CUFFT_Z2D, count) != CUFFT_SUCCESS)
        return done(qew_fail(ctx, QEW_ERR_CUDA, "line_statistics: cuFFT plan"));
    have_inv = true;
    if (cufftSetStream(fwd, ctx->stream) != CUFFT_SUCCESS ||
        cufftSetStream(inv, ctx->stream) != CUFFT_SUCCESS ||
        cufftExecD2Z(fwd, (cufftDoubleReal *)d_h, spec) != CUFFT_SUCCESS)
        return done(qew_fail(ctx, QEW_ERR_CUDA, "line_statistics: forward transform"));
    const long total = (long)count * nh;
    k_power<<<(unsigned)((total + kBS - 1) / kBS), kBS, 0, ctx->stream>>>(
        spec, total, nh, n, physical_size, d_q, d_psd);
    const qew_status st_power = qew_launch_check(ctx, "line_statistics_power");
    if (st_power != QEW_OK) return done(st_power);
    if (d_acf) {
        // cuFFT's Z2D may overwrite its input: spec is scratch, that is fine
        if (cufftExecZ2D(inv, spec, r) != CUFFT_SUCCESS)
            return done(qew_fail(ctx, QEW_ERR_CUDA, "line_statistics: inverse transform"));
        k_acf<<<(unsigned)((total + kBS - 1) / kBS), kBS, 0, ctx->stream>>>(r, count, n, nh,
                                                                           physical_size, d_ell,
                                                                           d_acf);
        const qew_status st = qew_launch_check(ctx, "line_statistics_acf");
        if (st != QEW_OK) return done(st);
    }
    return done(QEW_OK);
}

// The same from host arrays (h_h: count * n doubles; outputs as above, on the
// host), through stream-ordered device buffers.
extern "C" qew_status qew_line_statistics_host(qew_ctx *ctx, int count, const double *h_h, int n,
                                               double physical_size, double *h_ell,
                                               double *h_acf, double *h_q, double *h_psd) {
    QEW_RANGE();
    if (!ctx || count < 1 || !h_h || n < 2 || (!h_acf && !h_psd))
        return qew_fail(ctx, QEW_ERR_INVALID, "line_statistics_host: bad arguments");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nh = n / 2 + 1;
    const size_t hb = (size_t)count * n * sizeof(double);
    const size_t lb = (size_t)count * nh * sizeof(double);
    const size_t kb = (size_t)nh * sizeof(double);
    double *buf = nullptr;
    QEW_TRY(qew_alloc_async(ctx, (void **)&buf, hb + 2 * lb + 2 * kb + 5 * 256));
    auto align = [](size_t b) { return (b + 255) & ~size_t(255); };
    char *p = (char *)buf;
    double *d_h = (double *)p;
    p += align(hb);
    double *d_acf = (double *)p;
    p += align(lb);
    double *d_psd = (double *)p;
    p += align(lb);
    double *d_ell = (double *)p;
    p += align(kb);
    double *d_q = (double *)p;
    qew_status st = QEW_OK;
    if (cudaMemcpyAsync(d_h, h_h, hb, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        st = qew_fail(ctx, QEW_ERR_CUDA, "line_statistics_host: upload");
    if (st == QEW_OK)
        st = qew_line_statistics(ctx, count, d_h, n, physical_size, d_ell, d_acf, d_q, d_psd);
    struct Out {
        double *host;
        const double *dev;
        size_t bytes;
    } outs[4] = {{h_ell, d_ell, kb}, {h_acf, d_acf, lb}, {h_q, d_q, kb}, {h_psd, d_psd, lb}};
    for (const Out &o : outs)
        if (st == QEW_OK && o.host &&
            cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
            st = qew_fail(ctx, QEW_ERR_CUDA, "line_statistics_host: download");
    qew_free_async(buf, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && st == QEW_OK)
        st = qew_fail(ctx, QEW_ERR_CUDA, "line_statistics_host: synchronize");
    return st;
}
