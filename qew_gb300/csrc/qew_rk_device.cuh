// qew_rk_device.cuh -- device functions of the Rosso-Krauth construction
// (rosso_krauth.h:51-124): the single-site velocity and the nearest forward
// velocity zero (march, then bisect).
#pragma once

#include "qew_internal.cuh"

struct RkP {
    double dstep, max_advance, root_tol, sweep_tol, runaway;
    int max_sweeps;
};

inline RkP rkp_from(const qew_rk_params *rp) {
    return RkP{rp->dstep, rp->max_advance, rp->root_tol, rp->sweep_tol, rp->runaway, rp->max_sweeps};
}

// rk_site_velocity, rosso_krauth.h:51-82: exactly -gradient_i.
template <class Noise>
__device__ __forceinline__ double rk_site_velocity(const Noise &nz, int i, int n, double dx,
                                                   double lt, double f, int model, double hi,
                                                   double hl, double hr) {
    const int im = (i == 0) ? n - 1 : i - 1;
    const int ip = (i + 1 == n) ? 0 : i + 1;
    double line_force;
    if (model == QEW_MODEL_LINEAR) {
        line_force = -lt * (hl + hr - 2.0 * hi) / (dx * dx);
    } else {
        const double dhr = (hr - hi) / dx;
        const double dhl = (hi - hl) / dx;
        line_force = lt * (dhl / sqrt(1.0 + dhl * dhl) - dhr / sqrt(1.0 + dhr * dhr)) / dx;
    }
    const double xcl = (double)(im + i) * 0.5 * dx;
    const double hcl = (hl + hi) * 0.5;
    const double xcr = (double)(i + ip) * 0.5 * dx;
    const double hcr = (hi + hr) * 0.5;
    const double dvl = nz.dvdy(xcl, hcl);
    const double dvr = nz.dvdy(xcr, hcr);
    const double grad = dx * (line_force + 0.5 * (dvl + dvr) - f);
    return -grad;
}

// rk_forward_zero, rosso_krauth.h:88-124. The march is bounded by
// max_advance/dstep steps, the bisection by 60.
template <class Noise>
__device__ __forceinline__ double rk_forward_zero(const Noise &nz, int i, int n, double dx,
                                                  double lt, double f, int model, double hi,
                                                  double hl, double hr, const RkP &rp,
                                                  bool &found) {
    const double v0 = rk_site_velocity(nz, i, n, dx, lt, f, model, hi, hl, hr);
    if (v0 <= 0) {
        found = true;
        return hi;
    }
    double a = hi;
    double advanced = 0;
    while (advanced < rp.max_advance) {
        const double b = a + rp.dstep;
        const double vb = rk_site_velocity(nz, i, n, dx, lt, f, model, b, hl, hr);
        if (vb <= 0) {
            double lo = a, hc = b;
            for (int k = 0; k < 60 && (hc - lo) > rp.root_tol; ++k) {
                const double mid = 0.5 * (lo + hc);
                const double vm = rk_site_velocity(nz, i, n, dx, lt, f, model, mid, hl, hr);
                if (vm > 0)
                    lo = mid;
                else
                    hc = mid;
            }
            found = true;
            return 0.5 * (lo + hc);
        }
        a = b;
        advanced += rp.dstep;
    }
    found = false;
    return a;
}
