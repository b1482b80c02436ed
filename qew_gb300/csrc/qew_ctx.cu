// qew_ctx.cu -- context lifetime, error plumbing and scratch arena.
#include "qew_internal.cuh"

#include <cstring>
#include <new>

qew_status qew_fail(qew_ctx *ctx, qew_status s, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return s;
}

qew_status qew_scratch_reserve(qew_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return QEW_OK;
    // keep the work already queued on the old buffer safe before freeing it
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->scratch) cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    size_t want = bytes + (bytes >> 2);
    want = (want + 255) & ~size_t(255);
    if (cudaMalloc(&ctx->scratch, want) != cudaSuccess) {
        cudaGetLastError();
        return qew_fail(ctx, QEW_ERR_NOMEM, "scratch: cudaMalloc(%zu) failed", want);
    }
    ctx->scratch_bytes = want;
    return QEW_OK;
}

qew_status qew_launch_check(qew_ctx *ctx, const char *what, int k) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return qew_fail(ctx, QEW_ERR_CUDA, "launch %s: %s", what, cudaGetErrorString(e));
    ctx->launches += (uint64_t)k;
    return QEW_OK;
}

extern "C" {

const char *qew_status_string(qew_status s) {
    switch (s) {
    case QEW_OK: return "ok";
    case QEW_ERR_INVALID: return "invalid argument";
    case QEW_ERR_ODD_LENGTH: return "line length must be even for the red-black sweep";
    case QEW_ERR_CUDA: return "CUDA error";
    case QEW_ERR_NOMEM: return "out of device memory";
    case QEW_ERR_TIMEOUT: return "device-side wait timed out";
    case QEW_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

qew_status qew_ctx_create(int device, qew_ctx **out) {
    if (!out) return QEW_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return QEW_ERR_CUDA;
    }
    qew_ctx *ctx = new (std::nothrow) qew_ctx();
    if (!ctx) return QEW_ERR_NOMEM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&ctx->red_partials, sizeof(double) * 4 * QEW_RED_MAX_BLOCKS) != cudaSuccess ||
        cudaMalloc(&ctx->red_counter, sizeof(unsigned int) * 8) != cudaSuccess ||
        cudaMalloc(&ctx->red_out, sizeof(double) * 8) != cudaSuccess ||
        cudaMallocHost(&ctx->host_out, sizeof(double) * 8) != cudaSuccess ||
        cudaMemset(ctx->red_counter, 0, sizeof(unsigned int) * 8) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        qew_ctx_destroy(ctx);
        return QEW_ERR_CUDA;
    }
    *out = ctx;
    return QEW_OK;
}

qew_status qew_ctx_destroy(qew_ctx *ctx) {
    if (!ctx) return QEW_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->red_partials) cudaFree(ctx->red_partials);
    if (ctx->red_counter) cudaFree(ctx->red_counter);
    if (ctx->red_out) cudaFree(ctx->red_out);
    if (ctx->host_out) cudaFreeHost(ctx->host_out);
    if (ctx->scratch) cudaFree(ctx->scratch);
    delete ctx;
    return QEW_OK;
}

qew_status qew_ctx_set_stream(qew_ctx *ctx, void *cuda_stream) {
    if (!ctx) return QEW_ERR_INVALID;
    ctx->stream = (cudaStream_t)cuda_stream;
    return QEW_OK;
}

qew_status qew_ctx_synchronize(qew_ctx *ctx) {
    if (!ctx) return QEW_ERR_INVALID;
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

const char *qew_last_error(const qew_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

uint64_t qew_ctx_launch_count(const qew_ctx *ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
