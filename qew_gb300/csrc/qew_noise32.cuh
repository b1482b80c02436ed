// qew_noise32.cuh -- the FP32 split-index gather behind the FP64 Noise
// interface, for solvers that run their first iterations on FP32
// coefficients: the height is split into an integer cell and an FP32
// fraction (the only FP64 work is that split), the weights and the 16-tap
// sum are FP32, and the result is widened back to FP64. On a line with one
// point per field column, a field holding the x-filtered store (the x half of
// the stencil sum at every column midpoint) serves the edge midpoints with 4
// taps instead of 16.
#pragma once

#include "qew_internal.cuh"

__device__ __forceinline__ void bsw_value32(float t, float w[4]) {
    const float s6 = 1.0f / 6.0f;
    const float t2 = t * t, t3 = t2 * t, omt = 1.0f - t;
    w[0] = omt * omt * omt * s6;
    w[1] = (4.0f - 6.0f * t2 + 3.0f * t3) * s6;
    w[2] = (1.0f + 3.0f * t + 3.0f * t2 - 3.0f * t3) * s6;
    w[3] = t3 * s6;
}
__device__ __forceinline__ void bsw_deriv32(float t, float dw[4]) {
    const float t2 = t * t, omt = 1.0f - t;
    dw[0] = -0.5f * omt * omt;
    dw[1] = -2.0f * t + 1.5f * t2;
    dw[2] = 0.5f + t - 1.5f * t2;
    dw[3] = 0.5f * t2;
}

struct NoiseSplit32 {
    const float *__restrict__ coef;  // [ny][nx] FP32
    const float *__restrict__ edge;  // [ny][nx] x-filtered at e + 1/2 (xconst lines), or null
    int nx, ny;
    double dx, dy, inv_dx, inv_dy;
    bool dx_pow2, dy_pow2;
    bool xconst;  // as NoiseBSpline64::xconst
    float inv_dy_f;
    QEW_OOB_MEMBER

    __device__ __forceinline__ void loc_x(double x, int &ix, float &fx) const {
        double f;
        grid_locate(x, dx, inv_dx, dx_pow2, nx, ix, f);
        fx = (float)f;
    }
    __device__ __forceinline__ void loc_y(double y, int &iy, float &fy) const {
        double f;
        grid_locate(y, dy, inv_dy, dy_pow2, ny, iy, f);
        fy = (float)f;
    }
    __device__ __forceinline__ float taps(int ix, float fx, int iy, float fy, bool deriv) const {
        float wx[4], wy[4];
        bsw_value32(fx, wx);
        if (deriv)
            bsw_deriv32(fy, wy);
        else
            bsw_value32(fy, wy);
        float acc = 0.0f;
        if (ix >= 1 && ix <= nx - 3 && iy >= 1 && iy <= ny - 3) {
            // no wrap on either axis: one base pointer, taps at fixed offsets
            // (the same sum in the same order as below)
            const float *p = coef + ((size_t)(iy - 1) * (size_t)nx + (size_t)(ix - 1));
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const float *row = p + (size_t)b * (size_t)nx;
                const float r = wx[0] * QEW_LDGP(row, coef, (size_t)nx * ny, oob) +
                                wx[1] * QEW_LDGP(row + 1, coef, (size_t)nx * ny, oob) +
                                wx[2] * QEW_LDGP(row + 2, coef, (size_t)nx * ny, oob) +
                                wx[3] * QEW_LDGP(row + 3, coef, (size_t)nx * ny, oob);
                acc += wy[b] * r;
            }
            return acc;
        }
        int xs[4], ys[4];
        wrap4(ix, nx, xs);
        wrap4(iy, ny, ys);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float *row = coef + (size_t)ys[b] * (size_t)nx;
            const float r = wx[0] * QEW_LDGP(row + xs[0], coef, (size_t)nx * ny, oob) +
                            wx[1] * QEW_LDGP(row + xs[1], coef, (size_t)nx * ny, oob) +
                            wx[2] * QEW_LDGP(row + xs[2], coef, (size_t)nx * ny, oob) +
                            wx[3] * QEW_LDGP(row + xs[3], coef, (size_t)nx * ny, oob);
            acc += wy[b] * r;
        }
        return acc;
    }
    // The column sum at the midpoint of edge e from the x-filtered store.
    __device__ __forceinline__ float taps_edge(int e, int iy, float fy, bool deriv) const {
        float wy[4];
        if (deriv)
            bsw_deriv32(fy, wy);
        else
            bsw_value32(fy, wy);
        float acc = 0.0f;
        if (iy >= 1 && iy <= ny - 3) {
            const float *p = edge + ((size_t)(iy - 1) * (size_t)nx + (size_t)e);
#pragma unroll
            for (int b = 0; b < 4; ++b)
                acc += wy[b] * QEW_LDGP(p + (size_t)b * (size_t)nx, edge, (size_t)nx * ny, oob);
            return acc;
        }
        int ys[4];
        wrap4(iy, ny, ys);
#pragma unroll
        for (int b = 0; b < 4; ++b)
            acc += wy[b] * QEW_LDGP(edge + (size_t)ys[b] * (size_t)nx + (size_t)e, edge,
                                    (size_t)nx * ny, oob);
        return acc;
    }
    __device__ __forceinline__ double value(double x, double y) const {
        int ix, iy;
        float fx, fy;
        loc_x(x, ix, fx);
        loc_y(y, iy, fy);
        return (double)taps(ix, fx, iy, fy, false);
    }
    __device__ __forceinline__ double dvdy(double x, double y) const {
        int ix, iy;
        float fx, fy;
        loc_x(x, ix, fx);
        loc_y(y, iy, fy);
        return (double)(taps(ix, fx, iy, fy, true) * inv_dy_f);
    }
    __device__ __forceinline__ double value_edge(int e, double xc, double y) const {
        if (!xconst || e + 1 >= nx) return value(xc, y);
        int iy;
        float fy;
        loc_y(y, iy, fy);
        return (double)(edge ? taps_edge(e, iy, fy, false) : taps(e, 0.5f, iy, fy, false));
    }
    __device__ __forceinline__ double dvdy_edge(int e, double xc, double y) const {
        if (!xconst || e + 1 >= nx) return dvdy(xc, y);
        int iy;
        float fy;
        loc_y(y, iy, fy);
        const float t = edge ? taps_edge(e, iy, fy, true) : taps(e, 0.5f, iy, fy, true);
        return (double)(t * inv_dy_f);
    }
    __device__ __forceinline__ void sample(double x, double y, double &v, double &a,
                                           double &b) const {
        v = value(x, y);
        a = 0.0;  // dV/dx is never consumed by the solvers
        b = dvdy(x, y);
    }
};

#ifdef QEW_BOUNDS_CHECK
__device__ __forceinline__ unsigned long long *qew_noise_oob(const NoiseSplit32 &nz) {
    return nz.oob;
}
#endif
__device__ __forceinline__ double noise_dvdy_edge(const NoiseSplit32 &nz, int e, double xc,
                                                  double y) {
    return nz.dvdy_edge(e, xc, y);
}
__device__ __forceinline__ double noise_value_edge(const NoiseSplit32 &nz, int e, double xc,
                                                   double y) {
    return nz.value_edge(e, xc, y);
}

static inline NoiseSplit32 make_split32(const qew_field *f, int n, double physical_size) {
    NoiseSplit32 nz;
    nz.coef = f->coef32;
    nz.nx = f->nx;
    nz.ny = f->ny;
    nz.dx = f->dx;
    nz.dy = f->dy;
    nz.inv_dx = 1.0 / f->dx;
    nz.inv_dy = 1.0 / f->dy;
    nz.dx_pow2 = qew_is_pow2(f->dx);
    nz.dy_pow2 = qew_is_pow2(f->dy);
    nz.xconst = (n > 0 && n == f->nx && physical_size == f->Lx && nz.dx_pow2);
    nz.edge = nz.xconst ? f->edge32 : nullptr;
    nz.inv_dy_f = (float)(1.0 / f->dy);
#ifdef QEW_BOUNDS_CHECK
    nz.oob = qew_bounds_words();
#endif
    return nz;
}
