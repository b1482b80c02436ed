// qew_vec.cuh -- length-n vector kernels of the host-driven solver form
// (lbfgs.h:65-88 lbfgs_dot / lbfgs_max_abs / lbfgs_axpy and the small
// element-wise kernels of lbfgs_minimize), with deterministic reductions.
#pragma once

#include "qew_internal.cuh"

constexpr int kVecBS = 256;

inline int vec_red_blocks(int n) {
    int b = (n + kVecBS - 1) / kVecBS;
    return b < QEW_RED_MAX_BLOCKS ? (b > 0 ? b : 1) : QEW_RED_MAX_BLOCKS;
}

__device__ __forceinline__ double block_max(double v, double *s_warp) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) s_warp[w] = v;
    __syncthreads();
    double r = 0;
    if (w == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_down_sync(0xffffffffu, r, o));
    }
    __syncthreads();
    return r;
}

// NV simultaneous sums of f(i) (a functor filling v[NV]); deterministic
// (fixed partition, CTA trees, last-block final sum). MAX selects max-reduce.
template <class F, int NV, bool MAX>
__global__ void __launch_bounds__(kVecBS)
k_reduce(int n, F fn, double *partials, unsigned int *counter, double *out) {
    __shared__ double s_w[kVecBS / 32];
    __shared__ bool s_last;
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int i = blockIdx.x * kVecBS + threadIdx.x; i < n; i += gridDim.x * kVecBS) {
        double v[NV];
        fn(i, v);
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = MAX ? fmax(acc[k], v[k]) : acc[k] + v[k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const double b = MAX ? block_max(acc[k], s_w) : block_sum<kVecBS>(acc[k], s_w);
        if (threadIdx.x == 0) partials[k * QEW_RED_MAX_BLOCKS + blockIdx.x] = b;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double v = 0.0;
            for (int b = threadIdx.x; b < (int)gridDim.x; b += kVecBS) {
                const double p = __ldcg(partials + k * QEW_RED_MAX_BLOCKS + b);
                v = MAX ? fmax(v, p) : v + p;
            }
            const double t = MAX ? block_max(v, s_w) : block_sum<kVecBS>(v, s_w);
            if (threadIdx.x == 0) out[k] = t;
        }
        if (threadIdx.x == 0) *counter = 0u;
    }
}

struct DotF {
    const double *__restrict__ a;
    const double *__restrict__ b;
    __device__ __forceinline__ void operator()(int i, double v[1]) const { v[0] = a[i] * b[i]; }
};
struct AbsF {
    const double *__restrict__ a;
    __device__ __forceinline__ void operator()(int i, double v[1]) const { v[0] = fabs(a[i]); }
};
struct SumF {
    const double *__restrict__ a;
    __device__ __forceinline__ void operator()(int i, double v[1]) const { v[0] = a[i]; }
};
// lbfgs_sy (lbfgs.h:250-261): writes s = al*d, y = g_new - g and reduces
// s.y, s.s, y.y in one pass.
struct SyF {
    const double *__restrict__ d;
    const double *__restrict__ gn;
    const double *__restrict__ g;
    double *s_out;
    double *y_out;
    double al;
    __device__ __forceinline__ void operator()(int i, double v[3]) const {
        const double s = al * d[i];
        const double y = gn[i] - g[i];
        s_out[i] = s;
        y_out[i] = y;
        v[0] = s * y;
        v[1] = s * s;
        v[2] = y * y;
    }
};

static __global__ void k_axpy(int n, double c, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += c * x[i];
}
static __global__ void k_scale(int n, double c, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = c * x[i];
}
static __global__ void k_neg(int n, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = -y[i];
}
static __global__ void k_neg_copy(int n, const double *__restrict__ x, double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = -x[i];
}

// Host wrappers: launch a reduction and read the NV results back (synchronous).
template <class F, int NV, bool MAX>
qew_status vec_reduce(qew_ctx *ctx, int n, const F &fn, double *res) {
    k_reduce<F, NV, MAX><<<vec_red_blocks(n), kVecBS, 0, ctx->stream>>>(
        n, fn, ctx->red_partials, ctx->red_counter, ctx->red_out);
    QEW_TRY(qew_launch_check(ctx, "reduce"));
    QEW_CUDA(ctx, cudaMemcpyAsync(ctx->host_out, ctx->red_out, sizeof(double) * NV,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < NV; ++k) res[k] = ctx->host_out[k];
    return QEW_OK;
}
