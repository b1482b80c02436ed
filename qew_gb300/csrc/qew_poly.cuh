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

// Row cell and fraction of the midpoint of edge heights (he, hep), given
// a = he + hep: the exact bit path when it applies, else the reference's
// locate (filtered_noise.h:80-92) on hc = a / 2.
__device__ __forceinline__ void poly_locate(double a, int ky, double half_inv_dy,
                                            const NoiseBSpline64 &nz, int &iy, double &t) {
    const bool ok = (ky != kPolyNotPow2) ? poly_cell_exact(a, ky, nz.ny, iy, t)
                                          : poly_cell_exact(a * half_inv_dy, 0, nz.ny, iy, t);
    if (!ok) grid_locate(a * 0.5, nz.dy, nz.inv_dy, nz.dy_pow2, nz.ny, iy, t);
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
