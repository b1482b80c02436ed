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
#include "qew_philox.cuh"
#include "qew_poly.cuh"

#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <random>
#include <vector>

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

// E[j][e] = sum_a w_a(1/2) c[j][(e - 1 + a) mod nx], FP64 sum rounded once to
// FP32: the x part of the cubic B-spline sum (filtered_noise.h:33-44 at t = 1/2,
// where the weights are 1/48, 23/48, 23/48, 1/48) at the midpoint of every
// column pair; c is [ny][nx], x fastest.
__global__ void k_edge_fp32(const double *__restrict__ c, float *__restrict__ out, int nx, int ny) {
    const double w0 = 1.0 / 48.0, w1 = 23.0 / 48.0;
    for (int j = blockIdx.y; j < ny; j += gridDim.y) {
        const double *row = c + (size_t)j * (size_t)nx;
        float *o = out + (size_t)j * (size_t)nx;
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nx; e += gridDim.x * blockDim.x) {
            const int em = (e == 0) ? nx - 1 : e - 1;
            const int ep = (e + 1 == nx) ? 0 : e + 1;
            const int ep2 = (ep + 1 == nx) ? 0 : ep + 1;
            o[e] = (float)(w0 * row[em] + w1 * row[e] + w1 * row[ep] + w0 * row[ep2]);
        }
    }
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

// ---- synthetic field generation on the device ----
// White noise w[i][j] ~ N(0,1) from the Philox stream (seed, counter (pair of
// j, row i)), then a periodic Gaussian filter of std xi cells along each axis
// (the real-space form of exp(-(2 pi xi f)^2 / 2) in Fourier space; taps to
// |k| <= ceil(5 xi), normalised so the sum of squared taps is 1), in the
// reference's host layout [nx][ny].
__global__ void k_white_noise(double *w, int nx, int ny, uint64_t seed) {
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int pairs = (ny + 1) / 2;
    if (tid >= (long)nx * pairs) return;
    const int i = (int)(tid / pairs), jp = (int)(tid % pairs);
    double z0, z1;
    philox_normal_pair(seed, (uint64_t)i, (uint32_t)jp, z0, z1);
    w[(size_t)i * ny + 2 * jp] = z0;
    if (2 * jp + 1 < ny) w[(size_t)i * ny + 2 * jp + 1] = z1;
}

// out[i][j] = sum_k taps[k] * in[(i + k - R) mod nx][j]   (axis 0), or along j (axis 1).
__global__ void k_gauss_conv(const double *__restrict__ in, double *__restrict__ out, int nx,
                             int ny, const double *__restrict__ taps, int R, int axis) {
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (tid >= (long)nx * ny) return;
    const int i = (int)(tid / ny), j = (int)(tid % ny);
    double acc = 0.0;
    for (int k = -R; k <= R; ++k) {
        const double t = taps[k + R];
        if (axis == 0)
            acc += t * in[(size_t)pmod((long)i + k, nx) * ny + j];
        else
            acc += t * in[(size_t)i * ny + pmod((long)j + k, ny)];
    }
    out[tid] = acc;
}

__global__ void k_scale_inplace(double *a, size_t n, const double *scale) {
    const double s = *scale;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        a[k] *= s;
}

// Population mean and std of n values -> scale = amplitude / std (one CTA).
__global__ void k_std_scale(const double *__restrict__ a, size_t n, double amplitude,
                            double *scale) {
    __shared__ double s_w[32];
    double s1 = 0.0;
    for (size_t k = threadIdx.x; k < n; k += blockDim.x) s1 += a[k];
    s1 = block_sum<1024>(s1, s_w);
    __shared__ double s_mean;
    if (threadIdx.x == 0) s_mean = s1 / (double)n;
    __syncthreads();
    const double mean = s_mean;
    double s2 = 0.0;
    for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
        const double d = a[k] - mean;
        s2 += d * d;
    }
    s2 = block_sum<1024>(s2, s_w);
    if (threadIdx.x == 0) *scale = amplitude / sqrt(s2 / (double)n);
}

// Real part of the inverse transform times 1/(nx ny) (the backward
// normalisation of kokkos-fft and numpy's ifft2).
__global__ void k_real_part(const cufftDoubleComplex *__restrict__ b, size_t n, double inv_n,
                            double *__restrict__ out) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        out[k] = b[k].x * inv_n;
}

// numpy fftfreq(n)[k] in cycles per sample (filtered_noise.cpp:18-21).
double fft_freq(int k, int n) {
    const int ks = (k < (n + 1) / 2) ? k : k - n;
    return (double)ks / (double)n;
}

std::vector<double> gauss_taps(double xi, int &R) {
    R = (xi > 0) ? (int)ceil(5.0 * xi) : 0;
    std::vector<double> t(2 * R + 1);
    double s2 = 0.0;
    for (int k = -R; k <= R; ++k) {
        const double v = (xi > 0) ? exp(-0.5 * (double)k * k / (xi * xi)) : 1.0;
        t[k + R] = v;
        s2 += v * v;
    }
    for (double &v : t) v /= sqrt(s2);
    return t;
}

qew_status field_build(qew_ctx *ctx, const double *src, bool src_on_device, int nx,
                       int ny, double Lx, double Ly, int store, qew_field **out) {
    if (!ctx || !out || !src || nx <= 0 || ny <= 0 || !(Lx > 0) || !(Ly > 0) ||
        (store & (QEW_STORE_FP64 | QEW_STORE_FP32)) == 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create: bad arguments");
    if ((store & QEW_STORE_FP32_EDGE) && !(store & QEW_STORE_FP32))
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create: QEW_STORE_FP32_EDGE needs QEW_STORE_FP32");
    if ((store & QEW_STORE_FP64_POLY) && !(store & QEW_STORE_FP64))
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create: QEW_STORE_FP64_POLY needs QEW_STORE_FP64");
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
    f->stream = ctx->stream;
    auto cleanup = [&](qew_status s) {
        qew_free_async(tmp, ctx->stream);
        qew_free_async(c64, ctx->stream);
        qew_free_async(f->coef32, ctx->stream);
        qew_free_async(f->edge32, ctx->stream);
        qew_free_async(f->poly64, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        delete f;
        return s;
    };
    if (qew_alloc_async(ctx, (void **)&tmp, N * sizeof(double)) != QEW_OK ||
        qew_alloc_async(ctx, (void **)&c64, N * sizeof(double)) != QEW_OK)
        return cleanup(QEW_ERR_NOMEM);
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
        if (qew_alloc_async(ctx, (void **)&f->coef32, N * sizeof(float)) != QEW_OK)
            return cleanup(QEW_ERR_NOMEM);
        const int blocks = ctx->num_sms * 8;
        k_to_fp32<<<blocks, 256, 0, ctx->stream>>>(c64, f->coef32, N);
        st = qew_launch_check(ctx, "to_fp32");
        if (st != QEW_OK) return cleanup(st);
    }
    if (store & QEW_STORE_FP32_EDGE) {
        if (qew_alloc_async(ctx, (void **)&f->edge32, N * sizeof(float)) != QEW_OK)
            return cleanup(QEW_ERR_NOMEM);
        const dim3 eg((unsigned)std::min((nx + 255) / 256, 64), (unsigned)std::min(ny, 65535));
        k_edge_fp32<<<eg, 256, 0, ctx->stream>>>(c64, f->edge32, nx, ny);
        st = qew_launch_check(ctx, "edge_fp32");
        if (st != QEW_OK) return cleanup(st);
    }
    if (store & QEW_STORE_FP64_POLY) {
        if (qew_alloc_async(ctx, (void **)&f->poly64, 4 * N * sizeof(double)) != QEW_OK)
            return cleanup(QEW_ERR_NOMEM);
        st = qew_poly_store_build(ctx, c64, nx, ny, f->dy, f->poly64);
        if (st != QEW_OK) return cleanup(st);
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field build: %s", cudaGetErrorString(e)));
    qew_free_async(tmp, ctx->stream);
    tmp = nullptr;
    if (store & QEW_STORE_FP64) {
        f->coef64 = c64;
    } else {
        qew_free_async(c64, ctx->stream);
    }
    c64 = nullptr;
    *out = f;
    return QEW_OK;
}

}  // namespace

extern "C" {

qew_status qew_field_create_from_host(qew_ctx *ctx, const double *h_field, int nx, int ny,
                                      double Lx, double Ly, int store_flags, qew_field **out) {
    QEW_RANGE();
    return field_build(ctx, h_field, false, nx, ny, Lx, Ly, store_flags, out);
}

qew_status qew_field_create_from_device(qew_ctx *ctx, const double *d_field, int nx, int ny,
                                        double Lx, double Ly, int store_flags, qew_field **out) {
    QEW_RANGE();
    return field_build(ctx, d_field, true, nx, ny, Lx, Ly, store_flags, out);
}

qew_status qew_field_create_generated(qew_ctx *ctx, int nx, int ny, double Lx, double Ly,
                                     double amplitude, double xi_x_cells, double xi_y_cells,
                                     uint64_t seed, int store_flags, qew_field **out) {
    QEW_RANGE();
    if (!ctx || !out || nx <= 0 || ny <= 0 || !(xi_x_cells >= 0) || !(xi_y_cells >= 0) ||
        xi_x_cells > 4096 || xi_y_cells > 4096 || !(amplitude > 0))
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create_generated: bad arguments");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)nx * ny;
    int Rx, Ry;
    const std::vector<double> tx = gauss_taps(xi_x_cells, Rx), ty = gauss_taps(xi_y_cells, Ry);
    double *w = nullptr, *t = nullptr, *taps = nullptr;
    auto cleanup = [&](qew_status s) {
        qew_free_async(w, ctx->stream);
        qew_free_async(t, ctx->stream);
        qew_free_async(taps, ctx->stream);
        return s;
    };
    if (qew_alloc_async(ctx, (void **)&w, N * sizeof(double)) != QEW_OK ||
        qew_alloc_async(ctx, (void **)&t, N * sizeof(double)) != QEW_OK ||
        qew_alloc_async(ctx, (void **)&taps, (tx.size() + ty.size() + 1) * sizeof(double)) != QEW_OK)
        return cleanup(QEW_ERR_NOMEM);
    double *tapx = taps, *tapy = taps + tx.size(), *scale = tapy + ty.size();
    cudaError_t e = cudaMemcpyAsync(tapx, tx.data(), tx.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tapy, ty.data(), ty.size() * sizeof(double), cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e != cudaSuccess) return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "%s", cudaGetErrorString(e)));
    const long pairs = (long)nx * ((ny + 1) / 2);
    k_white_noise<<<(unsigned)((pairs + 255) / 256), 256, 0, ctx->stream>>>(w, nx, ny, seed);
    const unsigned blocks = (unsigned)((N + 255) / 256);
    k_gauss_conv<<<blocks, 256, 0, ctx->stream>>>(w, t, nx, ny, tapy, Ry, 1);
    k_gauss_conv<<<blocks, 256, 0, ctx->stream>>>(t, w, nx, ny, tapx, Rx, 0);
    k_std_scale<<<1, 1024, 0, ctx->stream>>>(w, N, amplitude, scale);
    k_scale_inplace<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(w, N, scale);
    qew_status st = qew_launch_check(ctx, "field_generate", 5);
    if (st != QEW_OK) return cleanup(st);
    st = field_build(ctx, w, true, nx, ny, Lx, Ly, store_flags, out);
    return cleanup(st);
}

qew_status qew_field_create_seeded(qew_ctx *ctx, int nx, int ny, double Lx, double Ly,
                                  double amplitude, double xi_x, double xi_y, uint64_t seed,
                                  int store_flags, qew_field **out) {
    QEW_RANGE();
    if (!ctx || !out || nx <= 0 || ny <= 0 || !(Lx > 0) || !(Ly > 0) ||
        !std::isfinite(amplitude) || !std::isfinite(xi_x) || !std::isfinite(xi_y))
        return qew_fail(ctx, QEW_ERR_INVALID, "field_create_seeded: bad arguments");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)nx * ny;
    cufftDoubleComplex *spec = nullptr, *stage = nullptr;
    double *w = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    const int rows = std::max(1, std::min(nx, (1 << 20) / ny));  // host rows per upload
    const size_t chunk = (size_t)rows * ny;
    cudaEvent_t done[2] = {nullptr, nullptr};
    auto cleanup = [&](qew_status s) {
        cudaStreamSynchronize(ctx->stream);
        if (have_plan) cufftDestroy(plan);
        for (cudaEvent_t &e : done)
            if (e) cudaEventDestroy(e);
        if (stage) cudaFreeHost(stage);
        qew_free_async(spec, ctx->stream);
        qew_free_async(w, ctx->stream);
        return s;
    };
    if (qew_alloc_async(ctx, (void **)&spec, N * sizeof(cufftDoubleComplex)) != QEW_OK ||
        qew_alloc_async(ctx, (void **)&w, N * sizeof(double) + 256) != QEW_OK ||
        cudaMallocHost((void **)&stage, 2 * chunk * sizeof(cufftDoubleComplex)) != cudaSuccess)
        return cleanup(qew_fail(ctx, QEW_ERR_NOMEM, "field_create_seeded: out of memory"));
    for (cudaEvent_t &e : done)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field_create_seeded: event"));
    // Random unit phases masked to the correlation ellipse, drawn on the host in
    // the reference's order (filtered_noise.cpp:37-53: i over nx outer, j inner,
    // one draw per entry whether masked or not), uploaded in row chunks through
    // two pinned buffers so drawing overlaps the copies.
    const double two_pi = 2.0 * std::acos(-1.0);
    const double dx = Lx / nx, dy = Ly / ny;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> phase(0.0, two_pi);
    for (int i0 = 0, b = 0; i0 < nx; i0 += rows, b ^= 1) {
        const int i1 = std::min(nx, i0 + rows);
        cufftDoubleComplex *hs = stage + (size_t)b * chunk;
        if (cudaEventSynchronize(done[b]) != cudaSuccess)
            return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field_create_seeded: upload"));
        for (int i = i0; i < i1; ++i) {
            const double fx = fft_freq(i, nx) / dx;
            for (int j = 0; j < ny; ++j) {
                const double fy = fft_freq(j, ny) / dy;
                const double ph = phase(rng);
                cufftDoubleComplex a{0.0, 0.0};
                if (!((fx * xi_x) * (fx * xi_x) + (fy * xi_y) * (fy * xi_y) > 1.0))
                    a = cufftDoubleComplex{std::cos(ph), std::sin(ph)};
                hs[(size_t)(i - i0) * ny + j] = a;
            }
        }
        cudaError_t e = cudaMemcpyAsync(spec + (size_t)i0 * ny, hs,
                                        (size_t)(i1 - i0) * ny * sizeof(cufftDoubleComplex),
                                        cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaEventRecord(done[b], ctx->stream);
        if (e != cudaSuccess) return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "%s", cudaGetErrorString(e)));
    }
    if (cufftPlan2d(&plan, nx, ny, CUFFT_Z2Z) != CUFFT_SUCCESS)
        return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "cufftPlan2d Z2Z(%d, %d) failed", nx, ny));
    have_plan = true;
    if (cufftSetStream(plan, ctx->stream) != CUFFT_SUCCESS ||
        cufftExecZ2Z(plan, spec, spec, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return cleanup(qew_fail(ctx, QEW_ERR_CUDA, "field_create_seeded: inverse FFT failed"));
    double *scale = w + N;
    k_real_part<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(spec, N, 1.0 / (double)N, w);
    k_std_scale<<<1, 1024, 0, ctx->stream>>>(w, N, amplitude, scale);
    k_scale_inplace<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(w, N, scale);
    qew_status st = qew_launch_check(ctx, "field_seeded", 3);
    if (st != QEW_OK) return cleanup(st);
    return cleanup(field_build(ctx, w, true, nx, ny, Lx, Ly, store_flags, out));
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
    // the coefficients may be in use on any stream: wait for the device
    const bool held = f->coef64 || f->coef32 || f->edge32 || f->poly64;
    if (held) cudaDeviceSynchronize();
    qew_free_async(f->coef64, f->stream);
    qew_free_async(f->coef32, f->stream);
    qew_free_async(f->edge32, f->stream);
    qew_free_async(f->poly64, f->stream);
    if (held) cudaStreamSynchronize(f->stream);
    delete f;
    return QEW_OK;
}

// Release a field whose coefficients were only used on `stream`: frees in
// that stream's order, without waiting for the rest of the device.
void qew_field_release_on(qew_field *f, cudaStream_t stream) {
    if (!f) return;
    qew_free_async(f->coef64, stream);
    qew_free_async(f->coef32, stream);
    qew_free_async(f->edge32, stream);
    qew_free_async(f->poly64, stream);
    delete f;
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
