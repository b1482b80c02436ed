// qew_field.cu -- pinning-field handles: device-side periodic cubic B-spline
// prefilter, x-fastest FP64/FP32 coefficient storage, and point sampling.
//
// The reference builds coefficients with an FFT division
// (filtered_noise.cpp:92-136): c = IFFT2(FFT2(s) / (Kx (x) Ky)) with
// K[m] = 2/3 + cos(2 pi m/N)/3, i.e. the exact solve of the circulant system
// (1/6, 2/3, 1/6) * c = s along each axis. The same exact solve is done here
// by the separable recursive filter of the cubic B-spline (pole
// z1 = sqrt(3) - 2; M. Unser, IEEE Trans. Signal Process. 41 (1993)) with the
// periodic initial conditions written in closed form, so the result equals
// the FFT division up to rounding, for any nx, ny, in O(nx*ny) work.
#include "qew_internal.cuh"

#include <cmath>
#include <new>

namespace {

// Periodic cubic B-spline prefilter along one axis, in two out-of-place
// passes over chunks of kChunk samples so that every line is split over many
// threads: causal y[k] = s[k] + z y[k-1], anticausal w[k] = y[k] + z w[k+1],
// c = -6 z w. A chunk starts its recursion kWarm samples early (late, for the
// anticausal pass) from zero, reading the periodic neighbours: the neglected
// tail is z^kWarm ~ 5e-37 of the signal, so every output equals the exact
// periodic solve up to rounding, for any N (the warm-up wraps for short N).
// Lines are m = 0..M-1 at stride `lst`; samples at stride `st`; consecutive
// threads take consecutive lines so each step's accesses coalesce when
// lst == 1.
constexpr double kPole = -0.26794919243112270;  // sqrt(3) - 2
constexpr int kChunk = 256;
constexpr int kWarm = 64;

__device__ __forceinline__ int pmod(long k, int N) {
    long r = k % N;
    return (int)(r < 0 ? r + N : r);
}

__global__ void k_prefilter_causal(const double *__restrict__ in, double *__restrict__ out,
                                   int N, long st, int M, long lst) {
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int nchunks = (N + kChunk - 1) / kChunk;
    if (tid >= (long)M * nchunks) return;
    const int m = (int)(tid % M), c = (int)(tid / M);
    const double *a = in + (long)m * lst;
    double *b = out + (long)m * lst;
    const int k0 = c * kChunk, k1 = min(k0 + kChunk, N);
    double y = 0.0;
    for (int k = k0 - kWarm; k < k0; ++k) y = a[(long)pmod(k, N) * st] + kPole * y;
    for (int k = k0; k < k1; ++k) {
        y = a[(long)k * st] + kPole * y;
        b[(long)k * st] = y;
    }
}

__global__ void k_prefilter_anticausal(const double *__restrict__ in, double *__restrict__ out,
                                       int N, long st, int M, long lst) {
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int nchunks = (N + kChunk - 1) / kChunk;
    if (tid >= (long)M * nchunks) return;
    const int m = (int)(tid % M), c = (int)(tid / M);
    const double *a = in + (long)m * lst;
    double *b = out + (long)m * lst;
    const int k0 = c * kChunk, k1 = min(k0 + kChunk, N);
    const double gain = -6.0 * kPole;
    double w = 0.0;
    for (int k = k1 - 1 + kWarm; k >= k1; --k) w = a[(long)pmod(k, N) * st] + kPole * w;
    for (int k = k1 - 1; k >= k0; --k) {
        w = a[(long)k * st] + kPole * w;
        b[(long)k * st] = gain * w;
    }
}

qew_status prefilter_axis(qew_ctx *ctx, double *a, double *work, int N, long st, int M,
                          long lst) {
    const long threads = (long)M * ((N + kChunk - 1) / kChunk);
    const unsigned blocks = (unsigned)((threads + 255) / 256);
    k_prefilter_causal<<<blocks, 256, 0, ctx->stream>>>(a, work, N, st, M, lst);
    k_prefilter_anticausal<<<blocks, 256, 0, ctx->stream>>>(work, a, N, st, M, lst);
    return qew_launch_check(ctx, "prefilter", 2);
}

// [nx][ny] -> [ny][nx] through a 32x33 shared tile.
__global__ void k_transpose(const double *__restrict__ in, double *__restrict__ out,
                            int nx, int ny) {
    __shared__ double tile[32][33];
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = i0 + r, j = j0 + threadIdx.x;
        if (i < nx && j < ny) tile[r][threadIdx.x] = in[(size_t)i * ny + j];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int j = j0 + r, i = i0 + threadIdx.x;
        if (i < nx && j < ny) out[(size_t)j * nx + i] = tile[threadIdx.x][r];
    }
}

__global__ void k_to_fp32(const double *__restrict__ in, float *__restrict__ out, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        out[k] = (float)in[k];
}

template <class Noise>
__global__ void k_sample(Noise nz, const double *__restrict__ x, const double *__restrict__ y,
                         int m, double *v, double *dvdx, double *dvdy) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    double a, b, c;
    nz.sample(x[k], y[k], a, b, c);
    if (v) v[k] = a;
    if (dvdx) dvdx[k] = b;
    if (dvdy) dvdy[k] = c;
}

qew_status field_build(qew_ctx *ctx, const double *src, bool src_on_device, int nx,
                       int ny, double Lx, double Ly, int store, qew_field **out) {
    if (!ctx || !out || !src || nx <= 0 || ny <= 0 || !(Lx > 0) || !(Ly > 0) ||
        (store & (QEW_STORE_FP64 | QEW_STORE_FP32)) == 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create: bad arguments");
    // transposes tile 32 columns per grid row: keep both extents within the grid limit
    if (nx > 65535 * 32 || ny > 65535 * 32)
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create: nx and ny must be <= %d", 65535 * 32);
    *out = nullptr;
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)nx * ny;
    qew_field *f = new (std::nothrow) qew_field();
    if (!f) return QEW_ERR_NOMEM;
    f->kind = QEW_FIELD_BSPLINE;
    f->device = ctx->device;
    f->nx = nx;
    f->ny = ny;
    f->Lx = Lx;
    f->Ly = Ly;
    f->dx = Lx / nx;  // filtered_noise.cpp:87
    f->dy = Ly / ny;
    double *tmp = nullptr, *c64 = nullptr;
    auto cleanup = [&](qew_status s) {
        if (tmp) cudaFree(tmp);
        if (c64) cudaFree(c64);
        if (f->coef32) cudaFree(f->coef32);
        delete f;
        return s;
    };
    if (cudaMalloc(&tmp, N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c64, N * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(qew_fail(ctx, QEW_ERR_NOMEM, "field_create: cudaMalloc of %zu bytes", 2 * N * 8));
    }
    cudaError_t e = cudaMemcpyAsync(tmp, src, N * sizeof(double),
                                    src_on_device ? cudaMemcpyDeviceToDevice
                                                  : cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e != cudaSuccess) return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field upload: %s", cudaGetErrorString(e)));
    // x pass in the host layout (lines j, stride ny), transpose, y pass in
    // the x-fastest layout (lines i, stride nx); c64 doubles as the work
    // buffer of the first pass.
    qew_status st = prefilter_axis(ctx, tmp, c64, nx, ny, ny, 1);
    if (st != QEW_OK) return cleanup(st);
    k_transpose<<<dim3((ny + 31) / 32, (nx + 31) / 32), dim3(32, 8), 0, ctx->stream>>>(tmp, c64, nx, ny);
    st = qew_launch_check(ctx, "transpose");
    if (st != QEW_OK) return cleanup(st);
    st = prefilter_axis(ctx, c64, tmp, ny, nx, nx, 1);
    if (st != QEW_OK) return cleanup(st);
    if (store & QEW_STORE_FP32) {
        if (cudaMalloc(&f->coef32, N * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            f->coef32 = nullptr;
            return cleanup(qew_fail(ctx, QEW_ERR_NOMEM, "field_create: FP32 copy"));
        }
        const int blocks = ctx->num_sms * 8;
        k_to_fp32<<<blocks, 256, 0, ctx->stream>>>(c64, f->coef32, N);
        st = qew_launch_check(ctx, "to_fp32");
        if (st != QEW_OK) return cleanup(st);
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field build: %s", cudaGetErrorString(e)));
    cudaFree(tmp);
    tmp = nullptr;
    if (store & QEW_STORE_FP64) {
        f->coef64 = c64;
    } else {
        cudaFree(c64);
    }
    c64 = nullptr;
    *out = f;
    return QEW_OK;
}

}  // namespace

extern "C" {

qew_status qew_field_create_from_host(qew_ctx *ctx, const double *h_field, int nx, int ny,
                                      double Lx, double Ly, int store_flags, qew_field **out) {
    return field_build(ctx, h_field, false, nx, ny, Lx, Ly, store_flags, out);
}

qew_status qew_field_create_from_device(qew_ctx *ctx, const double *d_field, int nx, int ny,
                                        double Lx, double Ly, int store_flags, qew_field **out) {
    return field_build(ctx, d_field, true, nx, ny, Lx, Ly, store_flags, out);
}

qew_status qew_field_create_analytic(qew_ctx *ctx, int kind, double p0, double p1, double p2,
                                     qew_field **out) {
    if (!ctx || !out || kind < QEW_FIELD_ZERO || kind > QEW_FIELD_SINCOS)
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create_analytic: bad kind %d", kind);
    qew_field *f = new (std::nothrow) qew_field();
    if (!f) return QEW_ERR_NOMEM;
    f->kind = kind;
    f->device = ctx->device;
    f->p0 = p0;
    f->p1 = p1;
    f->p2 = p2;
    *out = f;
    return QEW_OK;
}

qew_status qew_field_destroy(qew_field *f) {
    if (!f) return QEW_OK;
    cudaSetDevice(f->device);
    if (f->coef64 || f->coef32) cudaDeviceSynchronize();
    if (f->coef64) cudaFree(f->coef64);
    if (f->coef32) cudaFree(f->coef32);
    delete f;
    return QEW_OK;
}

qew_status qew_field_get_coefficients(qew_ctx *ctx, const qew_field *f, double *h_coef) {
    if (!ctx || !f || !h_coef || f->kind != QEW_FIELD_BSPLINE || !f->coef64)
        return qew_fail(ctx, QEW_ERR_INVALID, "get_coefficients: no FP64 B-spline coefficients");
    const size_t N = (size_t)f->nx * f->ny;
    double *tmp = nullptr;
    if (cudaMalloc(&tmp, N * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return qew_fail(ctx, QEW_ERR_NOMEM, "get_coefficients: cudaMalloc");
    }
    // [ny][nx] -> [nx][ny] is the same transpose with the roles swapped
    k_transpose<<<dim3((f->nx + 31) / 32, (f->ny + 31) / 32), dim3(32, 8), 0, ctx->stream>>>(
        f->coef64, tmp, f->ny, f->nx);
    qew_status st = qew_launch_check(ctx, "transpose");
    if (st == QEW_OK) {
        cudaError_t e = cudaMemcpyAsync(h_coef, tmp, N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) st = qew_fail(ctx, QEW_ERR_CUDA, "get_coefficients: %s", cudaGetErrorString(e));
    }
    cudaFree(tmp);
    return st;
}

qew_status qew_field_sample(qew_ctx *ctx, const qew_field *f, const double *d_x, const double *d_y,
                            int m, double *d_v, double *d_dvdx, double *d_dvdy) {
    if (!ctx || !f || (m > 0 && (!d_x || !d_y)) || m < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "field_sample: bad arguments");
    if (m == 0) return QEW_OK;
    return qew_dispatch_noise(ctx, f, [&](auto nz) -> qew_status {
        k_sample<<<(m + 255) / 256, 256, 0, ctx->stream>>>(nz, d_x, d_y, m, d_v, d_dvdx, d_dvdy);
        return qew_launch_check(ctx, "sample");
    });
}

}  // extern "C"
