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

// rk_site_velocity, rosso_krauth.h:51-82: exactly -gradient_i. Every
// expression that a contraction could change (1 + s^2) is unfused, and the
// others round the same either way (2*hi and 0.5*x are exact), so with the
// reference-exact functor the velocity is the reference's bit for bit.
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
        line_force = lt *
                     (dhl / sqrt(__dadd_rn(1.0, __dmul_rn(dhl, dhl))) -
                      dhr / sqrt(__dadd_rn(1.0, __dmul_rn(dhr, dhr)))) /
                     dx;
    }
    const double xcl = (double)(im + i) * 0.5 * dx;
    const double hcl = (hl + hi) * 0.5;
    const double xcr = (double)(i + ip) * 0.5 * dx;
    const double hcr = (hi + hr) * 0.5;
    const double dvl = noise_dvdy_edge(nz, im, xcl, hcl);  // edge (im, i)
    const double dvr = noise_dvdy_edge(nz, i, xcr, hcr);   // edge (i, ip)
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

// rk_forward_zero evaluated by a group of G lanes (G = 2, 4, 8, 16 or 32; the
// G lanes of one aligned G-lane slice of the warp, `lane` = 0..G-1 within it,
// all with the same site and neighbours). It returns exactly what
// rk_forward_zero returns: every velocity it compares is computed from the
// same operands by the same code, and the search is replayed step by step
// from those comparisons; only the evaluations are spread over the lanes.
//   * march: lane j evaluates the point the serial loop reaches after j + 1
//     steps of a round (each lane redoes the round's additions of dstep, so
//     its point is the serial one bit for bit); the first lane with v <= 0
//     brackets the zero, as the serial loop would have found it;
//   * bisection: lane j (1 <= j < G) evaluates node j of the next
//     log2(G)-level subtree of midpoints (heap order, each node's interval
//     replayed from the root with the serial midpoint formula); the walk down
//     the subtree then applies the serial loop's test and update per level.
template <int G, class Noise>
__device__ __forceinline__ double rk_forward_zero_group(const Noise &nz, int i, int n, double dx,
                                                        double lt, double f, int model, double hi,
                                                        double hl, double hr, const RkP &rp,
                                                        bool &found, int lane, unsigned gmask) {
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0, "G must be a power of two <= 32");
    constexpr int kLevels = (G >= 32) ? 5 : (G >= 16) ? 4 : (G >= 8) ? 3 : (G >= 4) ? 2 : 1;
    const double v0 = rk_site_velocity(nz, i, n, dx, lt, f, model, hi, hl, hr);
    if (v0 <= 0) {
        found = true;
        return hi;
    }
    double a = hi, advanced = 0.0;
    double lo = 0.0, hc = 0.0;
    bool bracketed = false;
    // The serial march takes at most ceil(max_advance / dstep) steps
    // (validated on the host), so this loop ends.
    while (!bracketed) {
        // this lane's point: j + 1 serial steps from (a, advanced)
        double la = a, ladv = advanced, b = a;
        bool valid = true;
        for (int t = 0; t <= lane; ++t) {
            if (!(ladv < rp.max_advance)) {
                valid = false;
                break;
            }
            b = la + rp.dstep;
            if (t < lane) {
                la = b;
                ladv += rp.dstep;
            }
        }
        const double vb = valid ? rk_site_velocity(nz, i, n, dx, lt, f, model, b, hl, hr) : 1.0;
        const unsigned shift = (unsigned)(threadIdx.x & 31) & ~(unsigned)(G - 1);
        const unsigned okm = (__ballot_sync(gmask, valid) >> shift) & ((G == 32) ? ~0u : ((1u << G) - 1));
        const unsigned hitm = (__ballot_sync(gmask, valid && vb <= 0) >> shift) &
                              ((G == 32) ? ~0u : ((1u << G) - 1));
        if (hitm) {
            const int j = __ffs(hitm) - 1;
            lo = __shfl_sync(gmask, la, j, G);
            hc = __shfl_sync(gmask, b, j, G);
            bracketed = true;
        } else {
            const bool all_ok = okm == ((G == 32) ? ~0u : ((1u << G) - 1));
            if (!all_ok) {
                // the march ran out of max_advance: the serial loop returns the
                // last point it stepped to (or a, when no step was possible)
                found = false;
                if (okm == 0) return a;
                const int last = 31 - __clz(okm);
                return __shfl_sync(gmask, b, last, G);
            }
            a = __shfl_sync(gmask, b, G - 1, G);
            advanced = __shfl_sync(gmask, ladv + rp.dstep, G - 1, G);
        }
    }
    // bisection: for (k = 0; k < 60 && (hc - lo) > root_tol; ++k)
    int k = 0;
    while (true) {
        // node `lane` (1..G-1) of the subtree rooted at the current interval
        double vm = 0.0;
        if (lane >= 1) {
            const int depth = 31 - __clz(lane);
            double l2 = lo, h2 = hc;
            for (int d = depth - 1; d >= 0; --d) {
                const double mid = 0.5 * (l2 + h2);
                if ((lane >> d) & 1)
                    l2 = mid;
                else
                    h2 = mid;
            }
            vm = rk_site_velocity(nz, i, n, dx, lt, f, model, 0.5 * (l2 + h2), hl, hr);
        }
        int node = 1;
        bool done = false;
        for (int level = 0; level < kLevels; ++level) {
            if (!(k < 60 && (hc - lo) > rp.root_tol)) {
                done = true;
                break;
            }
            const double mid = 0.5 * (lo + hc);
            const double v = __shfl_sync(gmask, vm, node, G);
            if (v > 0) {
                lo = mid;
                node = 2 * node + 1;
            } else {
                hc = mid;
                node = 2 * node;
            }
            ++k;
        }
        if (done || !(k < 60 && (hc - lo) > rp.root_tol)) break;
    }
    found = true;
    return 0.5 * (lo + hc);
}

// rk_site_velocity evaluated by a lane pair (lanes `lane` = 0 and 1 of an
// aligned pair, same site and heights): each lane gathers one of the two edge
// midpoints, the other one's value comes by shuffle, and both finish the
// same expression -- the value is rk_site_velocity's bit for bit.
template <class Noise>
__device__ __forceinline__ double rk_site_velocity_pair(const Noise &nz, int i, int n, double dx,
                                                        double lt, double f, int model, double hi,
                                                        double hl, double hr, int lane,
                                                        unsigned pmask) {
    const int im = (i == 0) ? n - 1 : i - 1;
    const int ip = (i + 1 == n) ? 0 : i + 1;
    double line_force;
    if (model == QEW_MODEL_LINEAR) {
        line_force = -lt * (hl + hr - 2.0 * hi) / (dx * dx);
    } else {
        const double dhr = (hr - hi) / dx;
        const double dhl = (hi - hl) / dx;
        line_force = lt *
                     (dhl / sqrt(__dadd_rn(1.0, __dmul_rn(dhl, dhl))) -
                      dhr / sqrt(__dadd_rn(1.0, __dmul_rn(dhr, dhr)))) /
                     dx;
    }
    const double xc = lane ? (double)(i + ip) * 0.5 * dx : (double)(im + i) * 0.5 * dx;
    const double hc = lane ? (hi + hr) * 0.5 : (hl + hi) * 0.5;
    const double mine = noise_dvdy_edge(nz, lane ? i : im, xc, hc);
    const double other = __shfl_xor_sync(pmask, mine, 1);
    const double dvl = lane ? other : mine;
    const double dvr = lane ? mine : other;
    const double grad = dx * (line_force + 0.5 * (dvl + dvr) - f);
    return -grad;
}

// rk_forward_zero with every velocity evaluated by a lane pair
// (rk_site_velocity_pair): the serial march and bisection, run identically by
// both lanes, with each evaluation's two gathers side by side. Same result as
// rk_forward_zero.
template <class Noise>
__device__ __forceinline__ double rk_forward_zero_pair(const Noise &nz, int i, int n, double dx,
                                                       double lt, double f, int model, double hi,
                                                       double hl, double hr, const RkP &rp,
                                                       bool &found, int lane, unsigned pmask) {
    const double v0 = rk_site_velocity_pair(nz, i, n, dx, lt, f, model, hi, hl, hr, lane, pmask);
    if (v0 <= 0) {
        found = true;
        return hi;
    }
    double a = hi;
    double advanced = 0;
    while (advanced < rp.max_advance) {
        const double b = a + rp.dstep;
        const double vb = rk_site_velocity_pair(nz, i, n, dx, lt, f, model, b, hl, hr, lane, pmask);
        if (vb <= 0) {
            double lo = a, hc = b;
            for (int k = 0; k < 60 && (hc - lo) > rp.root_tol; ++k) {
                const double mid = 0.5 * (lo + hc);
                const double vm =
                    rk_site_velocity_pair(nz, i, n, dx, lt, f, model, mid, hl, hr, lane, pmask);
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
