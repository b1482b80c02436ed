// qew_internal.cuh -- shared internals of the GB300 qEW library: context and
// field handles, error plumbing, and the device-side Noise functors.
//
// Noise functors mirror the reference's `Noise` concept (qew_model.h:14-17,
// 31-48): a copyable, device-callable object with value / dV/dy / full
// sample. NoiseBSpline64 restates DeviceNoise (filtered_noise.h:67-177) on an
// x-fastest coefficient array, keeping the reference's exact coordinate
// arithmetic (x/dx, periodic fold, floor) so the cell index and fraction are
// bit-identical to the reference's; only the weight polynomials use
// multiplications by 1/6 where the reference divides (a <= 1 ulp change).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/qew_gpu.h"
#include "qew_nvtx.cuh"

// ---------------------------------------------------------------- handles
struct qew_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // reduction scratch: per-block partials + a self-resetting ticket counter
    double *red_partials = nullptr;  // QEW_RED_MAX_BLOCKS * 4 doubles
    unsigned int *red_counter = nullptr;
    double *red_out = nullptr;       // 8 doubles of device results
    double *host_out = nullptr;      // pinned 8 doubles
    // general scratch arena (grown on demand, never shrunk)
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    uint64_t launches = 0;
    // upper bound on the warps of this context's persistent (cooperative)
    // kernels; 0 = every resident slot of the GPU. Contexts that share the GPU
    // (the server's workers) take a share each.
    int warp_cap = 0;
    // grid-barrier limits of this context's cooperative kernels: polls before
    // a wait gives up, and a CTA that skips its arrival (-1: none; a fault
    // that tests inject to make the waits run out)
    long long barrier_polls = 1LL << 26;
    int barrier_skip = -1;
    // launch-shape autotuning (qew_tune.cuh): on by default; tune_force[k]
    // >= 0 fixes kernel k's candidate (kernel ids of qew_tune.cuh)
    int autotune = 1;
    int tune_force[4] = {-1, -1, -1, -1};
    std::string last_error;
    // copy streams and slot events of the host-buffer batch pipeline
    // (created on first use)
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t ev_in[3] = {}, ev_comp[3] = {}, ev_out[3] = {}, ev_start = nullptr;
};

struct qew_field {
    int kind = QEW_FIELD_BSPLINE;
    int device = 0;
    int nx = 0, ny = 0;
    double Lx = 0, Ly = 0, dx = 1, dy = 1;
    double p0 = 0, p1 = 0, p2 = 0;
    double *coef64 = nullptr;  // [ny][nx], x fastest
    float *coef32 = nullptr;   // [ny][nx], x fastest
    float *edge32 = nullptr;   // [ny][nx]: coefficients filtered along x at e + 1/2
    double *poly64 = nullptr;  // [ny][nx][4]: FP64 cell polynomials of the x-filtered field
    cudaStream_t stream = nullptr;  // stream the coefficients were allocated on
};

#define QEW_RED_MAX_BLOCKS 1024

// Records the message on ctx (if any) and returns the status.
qew_status qew_fail(qew_ctx *ctx, qew_status s, const char *fmt, ...);
// Stream-ordered device allocation on ctx's stream (no device-wide sync).
qew_status qew_alloc_async(qew_ctx *ctx, void **p, size_t bytes);
void qew_free_async(void *p, cudaStream_t stream);
// Ensures ctx->scratch holds at least `bytes` (256-byte aligned base).
qew_status qew_scratch_reserve(qew_ctx *ctx, size_t bytes);
// Checks the last launch; bumps the launch counter by `k`.
qew_status qew_launch_check(qew_ctx *ctx, const char *what, int k = 1);

#define QEW_CUDA(ctx, call)                                                  \
    do {                                                                     \
        cudaError_t e__ = (call);                                            \
        if (e__ != cudaSuccess)                                              \
            return qew_fail((ctx), QEW_ERR_CUDA, "%s: %s", #call,            \
                            cudaGetErrorString(e__));                        \
    } while (0)

#define QEW_TRY(expr)                                                        \
    do {                                                                     \
        qew_status s__ = (expr);                                             \
        if (s__ != QEW_OK) return s__;                                       \
    } while (0)

// ------------------------------------------------------ bounds-check build
// Built with -DQEW_BOUNDS_CHECK (qew_gb300/build.py bounds_check=True), every
// field gather and the gradient kernels' shared-memory indices are checked:
// an index outside its array is counted in mapped host words (count, first
// index, its bound, source line; qew_bounds_check_report reads them) and
// clamped into range, so the access stays in bounds. The normal build
// compiles the bare accesses: these macros discard their check arguments.
// QEW_LDGP takes the pointer itself (the normal build's address arithmetic
// is then the unchecked code's, register for register) and the array's base.
#ifdef QEW_BOUNDS_CHECK
// Device address of the four mapped host words (allocated on first use).
unsigned long long *qew_bounds_words();
__device__ __forceinline__ long long qew_bc(long long i, long long n, unsigned long long *w,
                                            int line) {
    if (i >= 0 && i < n) return i;
    if (w && atomicAdd(w, 1ull) == 0ull) {
        w[1] = (unsigned long long)i;
        w[2] = (unsigned long long)n;
        w[3] = (unsigned long long)line;
    }
    return i < 0 ? 0 : (n > 0 ? n - 1 : 0);
}
template <class T>
__device__ __forceinline__ T qew_ldg_checked(const T *base, size_t off, size_t size,
                                             unsigned long long *w, int line) {
    return __ldg(base + (size_t)qew_bc((long long)off, (long long)size, w, line));
}
#define QEW_OOB_MEMBER unsigned long long *oob = nullptr;
#define QEW_IDX(i, n, w) ((int)qew_bc((i), (n), (w), __LINE__))
#define QEW_LDGP(ptr, base, size, w) \
    qew_ldg_checked((base), (size_t)((ptr) - (base)), (size), (w), __LINE__)
#define QEW_OOB_PARAMS , size_t oob_n, unsigned long long *oob
#define QEW_OOB_ARGS(n, w) , (n), (w)
#else
#define QEW_OOB_MEMBER
#define QEW_IDX(i, n, w) (i)
#define QEW_LDGP(ptr, base, size, w) __ldg(ptr)
#define QEW_OOB_PARAMS
#define QEW_OOB_ARGS(n, w)
#endif

// ------------------------------------------------------------ B-spline math
// Cubic B-spline weights for neighbours {i-1,i,i+1,i+2} at fraction t
// (filtered_noise.h:33-46), and their t-derivatives (filtered_noise.h:50-62).
__device__ __forceinline__ void bsw_value(double t, double w[4]) {
    const double s6 = 1.0 / 6.0;
    const double t2 = t * t, t3 = t2 * t, omt = 1.0 - t;
    w[0] = omt * omt * omt * s6;
    w[1] = (4.0 - 6.0 * t2 + 3.0 * t3) * s6;
    w[2] = (1.0 + 3.0 * t + 3.0 * t2 - 3.0 * t3) * s6;
    w[3] = t3 * s6;
}
__device__ __forceinline__ void bsw_deriv(double t, double dw[4]) {
    const double s6 = 1.0 / 6.0;
    const double t2 = t * t, omt = 1.0 - t;
    dw[0] = -omt * omt * 0.5;
    dw[1] = (-12.0 * t + 9.0 * t2) * s6;
    dw[2] = (3.0 + 6.0 * t - 9.0 * t2) * s6;
    dw[3] = 3.0 * t2 * s6;
}

// Physical -> grid coordinate along one axis with the periodic fold of
// DeviceNoise::locate (filtered_noise.h:80-92). Division by the spacing is
// replaced by a multiplication only when the spacing is a power of two
// (then both are exact); the fold is skipped when g is already in [0, n)
// (then floor(g/n) == 0 exactly, so the result is the same).
__device__ __forceinline__ void grid_locate(double x, double d, double inv_d,
                                            bool d_pow2, int n, int &ix,
                                            double &fx) {
    double g = d_pow2 ? x * inv_d : x / d;
    const double nd = (double)n;
    if (!(g >= 0.0 && g < nd)) g -= floor(g / nd) * nd;
    ix = (int)floor(g);
    if (ix >= n) {
        ix -= n;
        g -= nd;
    }
    fx = g - (double)ix;
    // Only a non-finite coordinate can leave [0, n) here; clamp so the
    // gather stays in bounds whatever the input (a no-op for finite x).
    ix = min(max(ix, 0), n - 1);
}

__device__ __forceinline__ void wrap4(int i, int n, int o[4]) {
    o[0] = (i == 0) ? n - 1 : i - 1;
    o[1] = i;
    o[2] = (i + 1 == n) ? 0 : i + 1;
    o[3] = (o[2] + 1 == n) ? 0 : o[2] + 1;
}

// True when d is a positive normal power of two: then x / d == x * (1/d)
// exactly, so a division by d may be replaced by a multiplication.
__host__ __device__ __forceinline__ bool dbl_is_pow2(double d) {
#ifdef __CUDA_ARCH__
    const long long b = __double_as_longlong(d);
#else
    long long b;
    memcpy(&b, &d, sizeof(b));
#endif
    return d > 0 && (b & 0x000FFFFFFFFFFFFFLL) == 0 && ((b >> 52) & 0x7FF) != 0;
}

// Line spacing dx = physical_size / n with exact shortcuts for its divisions.
struct LineDx {
    double dx, inv_dx, inv_dx2;
    bool pow2;
    __host__ __device__ __forceinline__ double div(double v) const {
        return pow2 ? v * inv_dx : v / dx;
    }
    __host__ __device__ __forceinline__ double div2(double v) const {  // v / (dx*dx)
        return pow2 ? v * inv_dx2 : v / (dx * dx);
    }
};
__host__ __device__ __forceinline__ LineDx make_line_dx(double physical_size, int n) {
    LineDx L;
    L.dx = physical_size / (double)n;
    L.inv_dx = 1.0 / L.dx;
    L.inv_dx2 = 1.0 / (L.dx * L.dx);
    L.pow2 = dbl_is_pow2(L.dx);
    return L;
}

// ------------------------------------------ FP64 cell-polynomial store
// (QEW_STORE_FP64_POLY): per (row cell j, column e) the cubic of the
// x-filtered field at x = e + 1/2 in the row fraction t, as
// {q0, q1, q2, v0} with dV/dy = q0 + t (q1 + t q2) and
// V = v0 + dy t (q0 + t (q1/2 + t q2/3)); qew_poly.cuh derives it.
// Marker for a row spacing that is not a power of two.
constexpr int kPolyNotPow2 = 1 << 20;

// 256-bit read-only load of one cell {q0, q1, q2, v0} (32-byte aligned).
__device__ __forceinline__ void poly_load4(const double *p, double &q0, double &q1, double &q2,
                                           double &v0) {
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
        : "=d"(q0), "=d"(q1), "=d"(q2), "=d"(v0)
        : "l"(p));
}
__device__ __forceinline__ void poly_load3(const double *p, double &q0, double &q1, double &q2) {
    double v0;
    poly_load4(p, q0, q1, q2, v0);
}

// g = a * 2^k. When g is finite, normal and in [0, ny) (ny < 2^30): iy =
// floor(g), t = g - iy exactly, and true; otherwise false (negative, >= ny,
// non-finite or subnormal heights take the reference's fold instead). Only
// integer operations on the bits of a.
__device__ __forceinline__ bool poly_cell_exact(double a, int k, int ny, int &iy, double &t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    const int ef = (int)(b >> 52);  // sign bit and biased exponent
    if (ef == 0) {                  // +0 (or a subnormal: the slow path)
        iy = 0;
        t = 0.0;
        return b == 0ull;
    }
    if (ef >= 2047) return false;   // negative, infinite or NaN
    const int eb = ef + k;          // biased exponent of g
    if (eb <= 0) return false;
    const int e = eb - 1023;
    if (e < 0) {                    // g in (0, 1): cell 0, t = g
        iy = 0;
        t = __longlong_as_double((long long)(b + ((unsigned long long)(long long)k << 52)));
        return true;
    }
    if (e > 29) return false;
    const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const int sh = 52 - e;          // 23 .. 52 fraction bits
    iy = (int)(m >> sh);
    if (iy >= ny) return false;
    const unsigned long long fb = m & ((1ull << sh) - 1ull);
    if (fb == 0ull) {
        t = 0.0;
        return true;
    }
    const int top = 63 - __clzll((long long)fb);  // leading bit of the fraction, < sh
    const unsigned long long mant = (fb << (52 - top)) & 0x000FFFFFFFFFFFFFull;
    t = __longlong_as_double((long long)(((unsigned long long)(top - sh + 1023) << 52) | mant));
    return true;
}

// dV/dy and V of a cell at fraction t.
__device__ __forceinline__ double poly_dvdy(double q0, double q1, double q2, double t) {
    return fma(fma(q2, t, q1), t, q0);
}
__device__ __forceinline__ double poly_value(double q0, double q1, double q2, double v0, double t,
                                             double dy) {
    const double third = 1.0 / 3.0;
    return fma(dy * t, fma(fma(q2 * third, t, 0.5 * q1), t, q0), v0);
}

// DeviceNoise on x-fastest FP64 coefficients.
struct NoiseBSpline64 {
    const double *__restrict__ coef;  // [ny][nx]
    int nx, ny;
    double dx, dy, inv_dx, inv_dy;
    bool dx_pow2, dy_pow2;
    // Set when the line has n == nx points over the field's length with a
    // power-of-two spacing: every edge midpoint but the wrap edge is then at
    // grid x = e + 1/2 exactly, so its cell is e and its x weights are those
    // of t = 1/2 (bit-identical to locating it).
    bool xconst;
    double wxc[4];
    // The field's FP64 cell-polynomial store when it serves this line (one
    // point per field column), else null; ky: y * 2^ky == y / dy exactly
    // (kPolyNotPow2 when dy is not a power of two).
    const double *__restrict__ poly;
    int ky;
    QEW_OOB_MEMBER

    // Row cell and fraction of height y: from y's bits when dy is a power of
    // two and y / dy lies in [0, ny), else the reference's locate.
    __device__ __forceinline__ void poly_row(double y, int &iy, double &t) const {
        const bool ok = (ky != kPolyNotPow2) ? poly_cell_exact(y, ky, ny, iy, t)
                                              : poly_cell_exact(y * inv_dy, 0, ny, iy, t);
        if (!ok) grid_locate(y, dy, inv_dy, dy_pow2, ny, iy, t);
    }

    __device__ __forceinline__ double c(int ix, int iy) const {
        ix = QEW_IDX(ix, nx, oob);
        iy = QEW_IDX(iy, ny, oob);
        return QEW_LDGP(coef + (size_t)iy * (size_t)nx + ix, coef, (size_t)nx * (size_t)ny, oob);
    }
    __device__ __forceinline__ void locate(double x, double y, int ixn[4],
                                           int iyn[4], double &fx,
                                           double &fy) const {
        int ix, iy;
        grid_locate(x, dx, inv_dx, dx_pow2, nx, ix, fx);
        grid_locate(y, dy, inv_dy, dy_pow2, ny, iy, fy);
        wrap4(ix, nx, ixn);
        wrap4(iy, ny, iyn);
    }
    // sample_value, filtered_noise.h:138-155
    __device__ __forceinline__ double value(double x, double y) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], wy[4];
        locate(x, y, ixn, iyn, fx, fy);
        bsw_value(fx, wx);
        bsw_value(fy, wy);
        double v = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) row += c(ixn[a], iyn[b]) * wy[b];
            v += wx[a] * row;
        }
        return v;
    }
    // sample_dy, filtered_noise.h:159-176
    __device__ __forceinline__ double dvdy(double x, double y) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], dwy[4];
        locate(x, y, ixn, iyn, fx, fy);
        bsw_value(fx, wx);
        bsw_deriv(fy, dwy);
        double dg = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) row += c(ixn[a], iyn[b]) * dwy[b];
            dg += wx[a] * row;
        }
        return dy_pow2 ? dg * inv_dy : dg / dy;
    }
    // dV/dy / V at the midpoint of edge e (xc its physical x). With the
    // cell-polynomial store: one 32-byte cell and two FMAs (the wrap edge,
    // e = nx - 1, is not at a half-integer column and keeps the 16 taps).
    __device__ __forceinline__ double dvdy_edge(int e, double xc, double y) const {
        if (poly && e + 1 < nx) {
            int iy;
            double t, q0, q1, q2;
            poly_row(y, iy, t);
            iy = QEW_IDX(iy, ny, oob);
            e = QEW_IDX(e, nx, oob);
            poly_load3(poly + ((size_t)iy * (size_t)nx + (size_t)e) * 4, q0, q1, q2);
            return poly_dvdy(q0, q1, q2, t);
        }
        if (!xconst || e + 1 >= nx) return dvdy(xc, y);
        int iy, xs[4], iyn[4];
        double fy, dwy[4];
        grid_locate(y, dy, inv_dy, dy_pow2, ny, iy, fy);
        wrap4(e, nx, xs);
        wrap4(iy, ny, iyn);
        bsw_deriv(fy, dwy);
        double dg = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) row += c(xs[a], iyn[b]) * dwy[b];
            dg += wxc[a] * row;
        }
        return dy_pow2 ? dg * inv_dy : dg / dy;
    }
    __device__ __forceinline__ double value_edge(int e, double xc, double y) const {
        if (poly && e + 1 < nx) {
            int iy;
            double t, q0, q1, q2, v0;
            poly_row(y, iy, t);
            iy = QEW_IDX(iy, ny, oob);
            e = QEW_IDX(e, nx, oob);
            poly_load4(poly + ((size_t)iy * (size_t)nx + (size_t)e) * 4, q0, q1, q2, v0);
            return poly_value(q0, q1, q2, v0, t, dy);
        }
        if (!xconst || e + 1 >= nx) return value(xc, y);
        int iy, xs[4], iyn[4];
        double fy, wy[4];
        grid_locate(y, dy, inv_dy, dy_pow2, ny, iy, fy);
        wrap4(e, nx, xs);
        wrap4(iy, ny, iyn);
        bsw_value(fy, wy);
        double v = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) row += c(xs[a], iyn[b]) * wy[b];
            v += wxc[a] * row;
        }
        return v;
    }
    // sample, filtered_noise.h:103-134
    __device__ __forceinline__ void sample(double x, double y, double &v,
                                           double &dvdx_,
                                           double &dvdy_) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], dwx[4], wy[4], dwy[4];
        locate(x, y, ixn, iyn, fx, fy);
        bsw_value(fx, wx);
        bsw_deriv(fx, dwx);
        bsw_value(fy, wy);
        bsw_deriv(fy, dwy);
        double vv = 0, gx = 0, gy = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0, row_dy = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const double cc = c(ixn[a], iyn[b]);
                row += cc * wy[b];
                row_dy += cc * dwy[b];
            }
            vv += wx[a] * row;
            gx += dwx[a] * row;
            gy += wx[a] * row_dy;
        }
        v = vv;
        dvdx_ = dx_pow2 ? gx * inv_dx : gx / dx;
        dvdy_ = dy_pow2 ? gy * inv_dy : gy / dy;
    }
};

// ------------------------------------------- reference-exact FP64 arithmetic
// The reference is ISO C++ evaluated expression by expression: every a*b+c is
// a rounded product and a rounded sum, every weight a true division by 6
// (filtered_noise.h:33-62). The __d*_rn intrinsics are never contracted into
// FMAs, so the functions below reproduce those operations bit for bit (the
// CPU oracle is compiled with -ffp-contract=off for the same reason).
__device__ __forceinline__ void bsw_value_ref(double t, double w[4]) {
    const double t2 = __dmul_rn(t, t);
    const double t3 = __dmul_rn(t2, t);
    const double omt = __dsub_rn(1.0, t);
    w[0] = __ddiv_rn(__dmul_rn(__dmul_rn(omt, omt), omt), 6.0);
    w[1] = __ddiv_rn(__dadd_rn(__dsub_rn(4.0, __dmul_rn(6.0, t2)), __dmul_rn(3.0, t3)), 6.0);
    w[2] = __ddiv_rn(__dsub_rn(__dadd_rn(__dadd_rn(1.0, __dmul_rn(3.0, t)), __dmul_rn(3.0, t2)),
                               __dmul_rn(3.0, t3)),
                     6.0);
    w[3] = __ddiv_rn(t3, 6.0);
}
__device__ __forceinline__ void bsw_deriv_ref(double t, double dw[4]) {
    const double t2 = __dmul_rn(t, t);
    const double omt = __dsub_rn(1.0, t);
    dw[0] = __ddiv_rn(__dmul_rn(-omt, omt), 2.0);
    dw[1] = __ddiv_rn(__dadd_rn(__dmul_rn(-12.0, t), __dmul_rn(9.0, t2)), 6.0);
    dw[2] = __ddiv_rn(__dsub_rn(__dadd_rn(3.0, __dmul_rn(6.0, t)), __dmul_rn(9.0, t2)), 6.0);
    dw[3] = __ddiv_rn(__dmul_rn(3.0, t2), 6.0);
}

// DeviceNoise with the reference's arithmetic exactly (filtered_noise.h:77-176):
// the same locate, true divisions, unfused sums in the reference's order.
struct NoiseBSpline64Ref {
    NoiseBSpline64 b;  // coefficients, extents and spacings (its xconst is not used)
    __device__ __forceinline__ double c(int ix, int iy) const { return b.c(ix, iy); }
    __device__ __forceinline__ double value(double x, double y) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], wy[4];
        b.locate(x, y, ixn, iyn, fx, fy);
        bsw_value_ref(fx, wx);
        bsw_value_ref(fy, wy);
        double v = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) row = __dadd_rn(row, __dmul_rn(c(ixn[a], iyn[k]), wy[k]));
            v = __dadd_rn(v, __dmul_rn(wx[a], row));
        }
        return v;
    }
    __device__ __forceinline__ double dvdy(double x, double y) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], dwy[4];
        b.locate(x, y, ixn, iyn, fx, fy);
        bsw_value_ref(fx, wx);
        bsw_deriv_ref(fy, dwy);
        double dg = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) row = __dadd_rn(row, __dmul_rn(c(ixn[a], iyn[k]), dwy[k]));
            dg = __dadd_rn(dg, __dmul_rn(wx[a], row));
        }
        return __ddiv_rn(dg, b.dy);
    }
    __device__ __forceinline__ void sample(double x, double y, double &v, double &dvdx_,
                                           double &dvdy_) const {
        int ixn[4], iyn[4];
        double fx, fy, wx[4], dwx[4], wy[4], dwy[4];
        b.locate(x, y, ixn, iyn, fx, fy);
        bsw_value_ref(fx, wx);
        bsw_deriv_ref(fx, dwx);
        bsw_value_ref(fy, wy);
        bsw_deriv_ref(fy, dwy);
        double vv = 0, gx = 0, gy = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double row = 0, row_dy = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double cc = c(ixn[a], iyn[k]);
                row = __dadd_rn(row, __dmul_rn(cc, wy[k]));
                row_dy = __dadd_rn(row_dy, __dmul_rn(cc, dwy[k]));
            }
            vv = __dadd_rn(vv, __dmul_rn(wx[a], row));
            gx = __dadd_rn(gx, __dmul_rn(dwx[a], row));
            gy = __dadd_rn(gy, __dmul_rn(wx[a], row_dy));
        }
        v = vv;
        dvdx_ = __ddiv_rn(gx, b.dx);
        dvdy_ = __ddiv_rn(gy, b.dy);
    }
};

// True for the functors whose callers must evaluate the rest of the model
// (elastic force, combine) with the reference's unfused arithmetic too.
template <class Noise>
struct noise_is_ref {
    static constexpr bool value = false;
};
template <>
struct noise_is_ref<NoiseBSpline64Ref> {
    static constexpr bool value = true;
};

// Analytic potentials of the reference's tests; value()/dvdy() go through
// sample() exactly like detail::noise_value/noise_dvdy (qew_model.h:31-46).
struct NoiseZero {
    __device__ __forceinline__ void sample(double, double, double &v,
                                           double &a, double &b) const {
        v = 0; a = 0; b = 0;
    }
    __device__ __forceinline__ double value(double, double) const { return 0; }
    __device__ __forceinline__ double dvdy(double, double) const { return 0; }
};
struct NoiseConst {
    double v0;
    __device__ __forceinline__ void sample(double, double, double &v,
                                           double &a, double &b) const {
        v = v0; a = 0; b = 0;
    }
    __device__ __forceinline__ double value(double, double) const { return v0; }
    __device__ __forceinline__ double dvdy(double, double) const { return 0; }
};
struct NoiseHarmonic {  // HarmonicWell{k, y0}
    double k, y0;
    __device__ __forceinline__ void sample(double, double y, double &v,
                                           double &a, double &b) const {
        const double d = y - y0;
        v = 0.5 * k * d * d; a = 0; b = k * d;
    }
    __device__ __forceinline__ double value(double, double y) const {
        const double d = y - y0;
        return 0.5 * k * d * d;
    }
    __device__ __forceinline__ double dvdy(double, double y) const {
        return k * (y - y0);
    }
};
struct NoiseWashboard {  // SinusoidNoise{A, k}: V = A cos(k y)
    double A, k;
    __device__ __forceinline__ void sample(double, double y, double &v,
                                           double &a, double &b) const {
        v = A * cos(k * y); a = 0; b = -A * k * sin(k * y);
    }
    __device__ __forceinline__ double value(double, double y) const {
        return A * cos(k * y);
    }
    __device__ __forceinline__ double dvdy(double, double y) const {
        return -A * k * sin(k * y);
    }
};
struct NoiseSinCos {  // AnalyticNoise{amp, kx, ky}
    double amp, kx, ky;
    __device__ __forceinline__ void sample(double x, double y, double &v,
                                           double &a, double &b) const {
        v = amp * sin(kx * x) * cos(ky * y);
        a = amp * kx * cos(kx * x) * cos(ky * y);
        b = -amp * ky * sin(kx * x) * sin(ky * y);
    }
    __device__ __forceinline__ double value(double x, double y) const {
        return amp * sin(kx * x) * cos(ky * y);
    }
    __device__ __forceinline__ double dvdy(double x, double y) const {
        return -amp * ky * sin(kx * x) * sin(ky * y);
    }
};

#ifdef QEW_BOUNDS_CHECK
// The error words a functor carries (none for the analytic potentials).
template <class Noise>
__device__ __forceinline__ unsigned long long *qew_noise_oob(const Noise &) { return nullptr; }
__device__ __forceinline__ unsigned long long *qew_noise_oob(const NoiseBSpline64 &nz) {
    return nz.oob;
}
__device__ __forceinline__ unsigned long long *qew_noise_oob(const NoiseBSpline64Ref &nz) {
    return nz.b.oob;
}
#endif

// Edge accessors for every functor: the B-spline one has its own fast path.
template <class Noise>
__device__ __forceinline__ double noise_dvdy_edge(const Noise &nz, int, double xc, double y) {
    return nz.dvdy(xc, y);
}
template <class Noise>
__device__ __forceinline__ double noise_value_edge(const Noise &nz, int, double xc, double y) {
    return nz.value(xc, y);
}
__device__ __forceinline__ double noise_dvdy_edge(const NoiseBSpline64 &nz, int e, double xc,
                                                  double y) {
    return nz.dvdy_edge(e, xc, y);
}
__device__ __forceinline__ double noise_value_edge(const NoiseBSpline64 &nz, int e, double xc,
                                                   double y) {
    return nz.value_edge(e, xc, y);
}

// Host helpers building the functors from a field handle.
static inline bool qew_is_pow2(double d) {
    int e;
    const double m = frexp(d, &e);
    return d > 0 && m == 0.5;
}
static inline NoiseBSpline64 make_bspline64(const qew_field *f, int n = 0,
                                            double physical_size = 0) {
    NoiseBSpline64 nz;
    nz.xconst = (n > 0 && n == f->nx && physical_size == f->Lx && qew_is_pow2(f->dx));
    {
        const double t = 0.5, s6 = 1.0 / 6.0, t2 = t * t, t3 = t2 * t, omt = 1.0 - t;
        nz.wxc[0] = omt * omt * omt * s6;  // the host twin of bsw_value(0.5)
        nz.wxc[1] = (4.0 - 6.0 * t2 + 3.0 * t3) * s6;
        nz.wxc[2] = (1.0 + 3.0 * t + 3.0 * t2 - 3.0 * t3) * s6;
        nz.wxc[3] = t3 * s6;
    }
    nz.coef = f->coef64;
    nz.nx = f->nx;
    nz.ny = f->ny;
    nz.dx = f->dx;
    nz.dy = f->dy;
    nz.inv_dx = 1.0 / f->dx;
    nz.inv_dy = 1.0 / f->dy;
    nz.dx_pow2 = qew_is_pow2(f->dx);
    nz.dy_pow2 = qew_is_pow2(f->dy);
    nz.poly = (f->poly64 && f->coef64 && n > 0 && n == f->nx && physical_size == f->Lx)
                  ? f->poly64
                  : nullptr;
    {
        int e;
        const double m = frexp(f->dy, &e);  // dy = m 2^e
        nz.ky = (f->dy > 0 && m == 0.5) ? 1 - e : kPolyNotPow2;
    }
#ifdef QEW_BOUNDS_CHECK
    nz.oob = qew_bounds_words();
#endif
    return nz;
}

// As qew_dispatch_noise, with the B-spline kind as NoiseBSpline64Ref (the
// reference's arithmetic bit for bit).
template <class Fn>
qew_status qew_dispatch_noise_ref(qew_ctx *ctx, const qew_field *f, Fn &&fn);

// Calls `fn(noise_functor)` with the functor matching the field's kind.
// Returns QEW_ERR_INVALID for an unknown kind or a B-spline field without
// FP64 coefficients. n / physical_size describe the line (0: unknown).
template <class Fn>
qew_status qew_dispatch_noise(qew_ctx *ctx, const qew_field *f, Fn &&fn, int n = 0,
                              double physical_size = 0) {
    switch (f->kind) {
    case QEW_FIELD_BSPLINE:
        if (!f->coef64)
            return qew_fail(ctx, QEW_ERR_INVALID,
                            "field has no FP64 coefficients (created without "
                            "QEW_STORE_FP64)");
        return fn(make_bspline64(f, n, physical_size));
    case QEW_FIELD_ZERO: return fn(NoiseZero{});
    case QEW_FIELD_CONST: return fn(NoiseConst{f->p0});
    case QEW_FIELD_HARMONIC: return fn(NoiseHarmonic{f->p0, f->p1});
    case QEW_FIELD_WASHBOARD: return fn(NoiseWashboard{f->p0, f->p1});
    case QEW_FIELD_SINCOS: return fn(NoiseSinCos{f->p0, f->p1, f->p2});
    default:
        return qew_fail(ctx, QEW_ERR_INVALID, "unknown field kind %d", f->kind);
    }
}

template <class Fn>
qew_status qew_dispatch_noise_ref(qew_ctx *ctx, const qew_field *f, Fn &&fn) {
    if (f->kind == QEW_FIELD_BSPLINE) {
        if (!f->coef64)
            return qew_fail(ctx, QEW_ERR_INVALID,
                            "field has no FP64 coefficients (created without "
                            "QEW_STORE_FP64)");
        return fn(NoiseBSpline64Ref{make_bspline64(f)});
    }
    return qew_dispatch_noise(ctx, f, fn);
}

// ------------------------------------------------------ block reductions
template <int BS>
__device__ __forceinline__ double block_sum(double v, double *s_warp) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) s_warp[w] = v;
    __syncthreads();
    double r = 0;
    if (w == 0) {
        r = (lane < BS / 32) ? s_warp[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}
