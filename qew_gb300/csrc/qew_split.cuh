// qew_split.cuh -- launch geometry of the FP32 split-index gather.
#pragma once

#include "qew_internal.cuh"

struct SplitGeom {
    const float *coef;  // [ny][nx] FP32 coefficients
    const float *edge;  // [ny][nx] x-filtered at e + 1/2 when same_grid and stored, else null
    int n, nx, ny;
    int same_grid;      // n == nx and physical_size == Lx: gx = e + 1/2 exactly
    double half_ratio;  // 0.5 * (physical_size / n) / dx_field (general case)
    double dy, inv_dy;  // FP64 height -> y-cells (drop-in input form)
    int dy_pow2;
    float inv_dy_f;       // d/dy of the interpolant: grid -> physical
    float dy_over_dx;     // arclength slope from a y-cell difference
    float lt_dy_over_dx2; // linear elastic force per y-cell of curvature
    float lt_over_dx;
    float dx_f;
    float f;
    int arc;
    QEW_OOB_MEMBER
};

SplitGeom qew_split_geom(const qew_field *f, int n, const qew_params *p);
