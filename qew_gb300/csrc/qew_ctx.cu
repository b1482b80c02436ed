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

qew_status qew_alloc_async(qew_ctx *ctx, void **p, size_t bytes) {
    *p = nullptr;
    if (cudaMallocAsync(p, bytes ? bytes : 1, ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return qew_fail(ctx, QEW_ERR_NOMEM, "cudaMallocAsync(%zu) failed", bytes);
    }
    return QEW_OK;
}

void qew_free_async(void *p, cudaStream_t stream) {
    if (p) cudaFreeAsync(p, stream);
}

qew_status qew_scratch_reserve(qew_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return QEW_OK;
    // stream-ordered: the old buffer is released after the work queued on it
    if (ctx->scratch) qew_free_async(ctx->scratch, ctx->stream);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    size_t want = bytes + (bytes >> 2);
    want = (want + 255) & ~size_t(255);
    QEW_TRY(qew_alloc_async(ctx, &ctx->scratch, want));
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

// Let the device's default memory pool keep up to 16 GiB of freed blocks for
// reuse (stream-ordered allocations of per-request buffers then stay cheap);
// the setting lives in this process only.
static bool keep_pool_cache(int device) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return true;
    uint64_t threshold = 16ull << 30;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    cudaGetLastError();
    return true;
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
        !keep_pool_cache(device) ||
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
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    for (cudaStream_t s : {ctx->copy_in, ctx->copy_out})
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (int k = 0; k < 3; ++k)
        for (cudaEvent_t e : {ctx->ev_in[k], ctx->ev_comp[k], ctx->ev_out[k]})
            if (e) cudaEventDestroy(e);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    delete ctx;
    return QEW_OK;
}

qew_status qew_ctx_set_stream(qew_ctx *ctx, void *cuda_stream) {
    if (!ctx) return QEW_ERR_INVALID;
    if ((cudaStream_t)cuda_stream != ctx->stream) {
        // the scratch arena is stream-ordered on the old stream: drain it first
        QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->stream = (cudaStream_t)cuda_stream;
    }
    return QEW_OK;
}

qew_status qew_ctx_set_barrier_limits(qew_ctx *ctx, long long max_polls, int skip_block) {
    if (!ctx || skip_block < -1) return QEW_ERR_INVALID;
    ctx->barrier_polls = max_polls > 0 ? max_polls : (1LL << 26);
    ctx->barrier_skip = skip_block;
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

#ifdef QEW_BOUNDS_CHECK
#include <mutex>
namespace {
std::mutex g_bounds_mu;
unsigned long long *g_bounds_host = nullptr, *g_bounds_dev = nullptr;
}  // namespace

unsigned long long *qew_bounds_words() {
    std::lock_guard<std::mutex> lock(g_bounds_mu);
    if (!g_bounds_host) {
        if (cudaHostAlloc((void **)&g_bounds_host, 4 * sizeof(unsigned long long),
                          cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&g_bounds_dev, g_bounds_host, 0) != cudaSuccess) {
            cudaGetLastError();
            g_bounds_host = nullptr;
            return nullptr;
        }
        memset(g_bounds_host, 0, 4 * sizeof(unsigned long long));
    }
    return g_bounds_dev;
}
#endif

extern "C" qew_status qew_bounds_check_report(long long out[4]) {
#ifdef QEW_BOUNDS_CHECK
    if (!out) return QEW_ERR_INVALID;
    qew_bounds_words();
    std::lock_guard<std::mutex> lock(g_bounds_mu);
    if (!g_bounds_host) return QEW_ERR_CUDA;
    cudaDeviceSynchronize();
    for (int k = 0; k < 4; ++k) {
        out[k] = (long long)__atomic_load_n(&g_bounds_host[k], __ATOMIC_ACQUIRE);
        g_bounds_host[k] = 0;
    }
    return QEW_OK;
#else
    (void)out;
    return QEW_ERR_UNSUPPORTED;
#endif
}
