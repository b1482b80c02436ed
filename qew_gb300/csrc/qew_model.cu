// qew_model.cu -- energy and gradient of the periodic line (qew_model.h).
//
// gradient: the reference runs two kernels, an edge pass writing dV/dy (and
// the arclength slope) of every edge to scratch and a per-site combine
// (qew_model.h:163-193). Here one kernel does both: each CTA computes the
// edges of its sites plus one halo edge into shared memory, then combines, so
// the per-edge scratch never touches HBM and one launch replaces two.
//
// objective: the per-edge energy (qew_model.h:61-83) reduced by a fixed
// grid-stride / warp-shuffle / CTA tree with a last-block final sum, so the
// result is bit-reproducible for a given n regardless of scheduling.
#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"
#include "qew_poly.cuh"

namespace {

constexpr int kGradBS = 256;
constexpr int kObjBS = 256;

int objective_blocks(int n) {
    int b = (n + kObjBS - 1) / kObjBS;
    return b < QEW_RED_MAX_BLOCKS ? (b > 0 ? b : 1) : QEW_RED_MAX_BLOCKS;
}

template <class At>
qew_status objective_impl(qew_ctx *ctx, const qew_field *field, const At &at, int n,
                          const qew_params *p, double *h_out) {
    if (!ctx || !field || !p || !h_out || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "objective: bad arguments");
    const LineDx dx = make_line_dx(p->physical_size, n);
    const int blocks = objective_blocks(n);
    QEW_TRY(qew_dispatch_noise(ctx, field, [&](auto nz) -> qew_status {
        k_objective<decltype(nz), At, kObjBS><<<blocks, kObjBS, 0, ctx->stream>>>(
            n, dx, p->line_tension, p->driving_force, p->model, nz, at, ctx->red_partials,
            ctx->red_counter, ctx->red_out);
        return qew_launch_check(ctx, "objective");
    }, n, p->physical_size));
    QEW_CUDA(ctx, cudaMemcpyAsync(ctx->host_out, ctx->red_out, sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *h_out = ctx->host_out[0];
    return QEW_OK;
}

// Device address of host memory that the GPU can reach directly (pinned or
// registered host memory, mapped into the device's address space), or null
// for pageable memory. Needs the context's device current.
const void *mapped_host_address(const void *ptr) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return a.devicePointer;
}

}  // namespace

// Host-buffer gradients without copies: when both host buffers are mapped
// (pinned) host memory, the kernels read the heights and write the
// gradients through the host link themselves (NVLink-C2C on Grace-based
// systems), so the transfer and the gather overlap inside one launch.
// QEW_ERR_UNSUPPORTED (nothing done) when either buffer is pageable or not
// 8-byte aligned.
static qew_status gradient_mapped(qew_ctx *ctx, const qew_field *field, int count,
                                  const double *h_h, int n, const qew_params *p, int precision,
                                  double *h_grad) {
    if (((uintptr_t)h_h | (uintptr_t)h_grad) & 7u) return QEW_ERR_UNSUPPORTED;
    const double *dh = (const double *)mapped_host_address(h_h);
    double *dg = (double *)mapped_host_address(h_grad);
    if (!dh || !dg) return QEW_ERR_UNSUPPORTED;
    QEW_TRY(qew_gradient_batch(ctx, field, count, dh, n, p, precision, dg));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

qew_status qew_gradient_enqueue(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                                const qew_params *p, int precision, double *d_grad) {
    if (!ctx || !field || !p || !d_h || !d_grad || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient: bad arguments");
    const LineDx dx = make_line_dx(p->physical_size, n);
    const int blocks = (n + kGradBS - 1) / kGradBS;
    if (precision == QEW_PREC_FP32_SPLIT) {
        if (field->kind != QEW_FIELD_BSPLINE || !field->coef32)
            return qew_fail(ctx, QEW_ERR_INVALID,
                            "gradient: FP32 split gather needs a B-spline field stored with QEW_STORE_FP32");
        return qew_gradient_split_enqueue(ctx, field, d_h, n, p, d_grad);
    }
    auto launch = [&](auto nz) -> qew_status {
        k_gradient<decltype(nz), kGradBS><<<blocks, kGradBS, 0, ctx->stream>>>(
            d_h, n, dx, p->line_tension, p->driving_force, p->model, nz, d_grad);
        return qew_launch_check(ctx, "gradient");
    };
    if (precision == QEW_PREC_FP64_REFERENCE) return qew_dispatch_noise_ref(ctx, field, launch);
    if (precision != QEW_PREC_FP64)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient: unknown precision %d", precision);
    // the cell-polynomial store, when it serves this line
    const qew_status s = qew_gradient_poly_enqueue(ctx, field, 1, d_h, n, p, d_grad);
    if (s != QEW_ERR_UNSUPPORTED) return s;
    return qew_dispatch_noise(ctx, field, launch, n, p->physical_size);
}

extern "C" {

qew_status qew_objective(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                         const qew_params *p, double *h_out) {
    QEW_RANGE();
    if (!d_h) return qew_fail(ctx, QEW_ERR_INVALID, "objective: null h");
    return objective_impl(ctx, field, LineAt{d_h}, n, p, h_out);
}

qew_status qew_objective_trial(qew_ctx *ctx, const qew_field *field, const double *d_x0,
                               const double *d_d, double alpha, int n, const qew_params *p,
                               double *h_out) {
    QEW_RANGE();
    if (!d_x0 || !d_d) return qew_fail(ctx, QEW_ERR_INVALID, "objective_trial: null input");
    return objective_impl(ctx, field, TrialAt{d_x0, d_d, alpha}, n, p, h_out);
}

qew_status qew_gradient(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                        const qew_params *p, double *d_grad) {
    QEW_RANGE();
    return qew_gradient_enqueue(ctx, field, d_h, n, p, QEW_PREC_FP64, d_grad);
}

qew_status qew_gradient_prec(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                             const qew_params *p, int precision, double *d_grad) {
    QEW_RANGE();
    return qew_gradient_enqueue(ctx, field, d_h, n, p, precision, d_grad);
}

qew_status qew_gradient_batch(qew_ctx *ctx, const qew_field *field, int count, const double *d_h,
                              int n, const qew_params *p, int precision, double *d_grad) {
    QEW_RANGE();
    if (!ctx || !field || !p || !d_h || !d_grad || n < 1 || count < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient_batch: bad arguments");
    if (count == 0) return QEW_OK;
    if (precision == QEW_PREC_FP64) {
        const qew_status s = qew_gradient_poly_enqueue(ctx, field, count, d_h, n, p, d_grad);
        if (s != QEW_ERR_UNSUPPORTED) return s;
    }
    for (int k = 0; k < count; ++k)
        QEW_TRY(qew_gradient_enqueue(ctx, field, d_h + (size_t)k * n, n, p, precision,
                                     d_grad + (size_t)k * n));
    return QEW_OK;
}

qew_status qew_gradient_host(qew_ctx *ctx, const qew_field *field, const double *h_h, int n,
                             const qew_params *p, int precision, double *h_grad) {
    QEW_RANGE();
    if (!ctx || !h_h || !h_grad || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient_host: bad arguments");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (const qew_status s = gradient_mapped(ctx, field, 1, h_h, n, p, precision, h_grad);
        s != QEW_ERR_UNSUPPORTED)
        return s;
    const size_t bytes = sizeof(double) * (size_t)n;
    QEW_TRY(qew_scratch_reserve(ctx, 2 * bytes + 256));
    double *d_h = (double *)ctx->scratch;
    double *d_g = d_h + (((size_t)n + 31) & ~size_t(31));
    QEW_CUDA(ctx, cudaMemcpyAsync(d_h, h_h, bytes, cudaMemcpyHostToDevice, ctx->stream));
    QEW_TRY(qew_gradient_enqueue(ctx, field, d_h, n, p, precision, d_g));
    QEW_CUDA(ctx, cudaMemcpyAsync(h_grad, d_g, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

// Lines k = 0..count-1 of h_h (n apart) through three device slots: the
// upload of line k, the gradient of line k-1 and the download of line k-2 run
// at the same time on three streams (copy_in, ctx->stream, copy_out), ordered
// by per-slot events, so the host link carries both directions at once.
qew_status qew_gradient_host_batch(qew_ctx *ctx, const qew_field *field, int count,
                                   const double *h_h, int n, const qew_params *p, int precision,
                                   double *h_grad) {
    QEW_RANGE();
    if (!ctx || !h_h || !h_grad || n < 1 || count < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient_host_batch: bad arguments");
    if (count == 0) return QEW_OK;
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (const qew_status s = gradient_mapped(ctx, field, count, h_h, n, p, precision, h_grad);
        s != QEW_ERR_UNSUPPORTED)
        return s;
    if (!ctx->copy_in) {
        QEW_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
        QEW_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
        QEW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_start, cudaEventDisableTiming));
        for (int s = 0; s < 3; ++s) {
            QEW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_in[s], cudaEventDisableTiming));
            QEW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_comp[s], cudaEventDisableTiming));
            QEW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_out[s], cudaEventDisableTiming));
        }
    }
    constexpr int S = 3;
    const size_t bytes = sizeof(double) * (size_t)n;
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    QEW_TRY(qew_scratch_reserve(ctx, 2 * S * npad * sizeof(double) + 256));
    double *dh[S], *dg[S];
    for (int s = 0; s < S; ++s) {
        dh[s] = (double *)ctx->scratch + (size_t)(2 * s) * npad;
        dg[s] = (double *)ctx->scratch + (size_t)(2 * s + 1) * npad;
    }
    // the copy streams start after everything already queued on ctx->stream
    QEW_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_in, ctx->ev_start, 0));
    QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_out, ctx->ev_start, 0));
    for (int k = 0; k < count; ++k) {
        const int s = k % S;
        if (k >= S) QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_in, ctx->ev_comp[s], 0));
        QEW_CUDA(ctx, cudaMemcpyAsync(dh[s], h_h + (size_t)k * n, bytes, cudaMemcpyHostToDevice,
                                      ctx->copy_in));
        QEW_CUDA(ctx, cudaEventRecord(ctx->ev_in[s], ctx->copy_in));
        QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_in[s], 0));
        if (k >= S) QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_out[s], 0));
        QEW_TRY(qew_gradient_enqueue(ctx, field, dh[s], n, p, precision, dg[s]));
        QEW_CUDA(ctx, cudaEventRecord(ctx->ev_comp[s], ctx->stream));
        QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_out, ctx->ev_comp[s], 0));
        QEW_CUDA(ctx, cudaMemcpyAsync(h_grad + (size_t)k * n, dg[s], bytes, cudaMemcpyDeviceToHost,
                                      ctx->copy_out));
        QEW_CUDA(ctx, cudaEventRecord(ctx->ev_out[s], ctx->copy_out));
    }
    // later work on ctx->stream (scratch reuse) follows the last download
    QEW_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_out[(count - 1) % S], 0));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->copy_out));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

}  // extern "C"
