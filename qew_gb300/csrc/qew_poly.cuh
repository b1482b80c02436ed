// qew_poly.cuh -- the FP64 cell-polynomial store and its device helpers.
//
// On a line with one point per field column (n == nx, physical size == Lx)
// every edge midpoint but the wrap edge sits at grid x = e + 1/2, where the
// x weights of the cubic B-spline are the constants w(1/2) = 1/48, 23/48,
// 23/48, 1/48 (filtered_noise.h:33-44 at t = 1/2). Along y, inside row cell
// j the interpolant is a cubic in the fraction t (filtered_noise.h:33-62):
// with E_b the x-filtered coefficients of rows j-1 .. j+2,
//   V(t)     = (E0 + 4 E1 + E2)/6 + t (E2 - E0)/2 + t^2 (E0 - 2 E1 + E2)/2
//              + t^3 (-E0 + 3 E1 - 3 E2 + E3)/6
//   dV/dt(t) = (E2 - E0)/2 + t (E0 - 2 E1 + E2) + t^2 (-E0 + 3 E1 - 3 E2 + E3)/2.
// The store keeps, per (row cell j, column e), four FP64 numbers
//   {q0, q1, q2, v0}:  dV/dy = q0 + t (q1 + t q2)   (q = dV/dt coefficients / dy)
//                      V     = v0 + dy t (q0 + t (q1/2 + t q2/3)),
// computed once in FP64 when the field is built. A gradient edge then reads
// one aligned 32-byte cell and evaluates two FMAs, where the reference's
// order (filtered_noise.h:159-176) reads 16 taps and forms 4 + 4 weights and
// 20 products. GB300 runs FP64 at 1/64 of its FP32 rate, so that FP64 work,
// not the memory traffic, is what bounds the plain FP64 gather.
//
// The row cell and fraction of an edge midpoint are found without FP64
// arithmetic when the field's row spacing is a power of two: the midpoint
// height in cells is (h_e + h_{e+1}) * 2^k exactly, and its floor and
// fraction are read off the bits of the FP64 sum (exact integer operations,
// the same numbers the reference's floor and subtraction give).
#pragma once

#include "qew_internal.cuh"

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

// Row cell and fraction of the midpoint of edge heights (he, hep), given
// a = he + hep: the exact bit path when it applies, else the reference's
// locate (filtered_noise.h:80-92) on hc = a / 2.
__device__ __forceinline__ void poly_locate(double a, int ky, double half_inv_dy,
                                            const NoiseBSpline64 &nz, int &iy, double &t) {
    const bool ok = (ky != kPolyNotPow2) ? poly_cell_exact(a, ky, nz.ny, iy, t)
                                          : poly_cell_exact(a * half_inv_dy, 0, nz.ny, iy, t);
    if (!ok) grid_locate(a * 0.5, nz.dy, nz.inv_dy, nz.dy_pow2, nz.ny, iy, t);
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

// Scale exponent k with (h_e + h_ep) * 2^k == ((h_e + h_ep) / 2) / dy exactly,
// or kPolyNotPow2.
static inline int poly_scale_exponent(double dy) {
    int e;
    const double m = frexp(dy, &e);  // dy = m 2^e, m in [0.5, 1)
    if (!(dy > 0) || m != 0.5) return kPolyNotPow2;
    return -1 - (e - 1);  // 1/(2 dy) = 2^(-1 - (e - 1))
}

// Builds the store of a field's FP64 coefficients c ([ny][nx], x fastest)
// into out ([ny][nx][4], 32-byte aligned), on ctx's stream.
qew_status qew_poly_store_build(qew_ctx *ctx, const double *c, int nx, int ny, double dy,
                                double *out);
// FP64 gradient of `count` lines (n apart) on the store; QEW_ERR_UNSUPPORTED
// (no error recorded) when the field holds no store or the line does not
// have one point per field column.
qew_status qew_gradient_poly_enqueue(qew_ctx *ctx, const qew_field *f, int count,
                                     const double *d_h, int n, const qew_params *p,
                                     double *d_grad);
// True when the store serves this line.
bool qew_poly_applies(const qew_field *f, int n, const qew_params *p);
