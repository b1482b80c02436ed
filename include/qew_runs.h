/*
 * qew_runs.h -- the reference's three production drivers over the GPU
 * handles of qew_gpu.h: static_sweep, dynamic_anneal and depinning_ramp
 * (qew_runs.h:45-243 of the reference), with the same configuration fields,
 * defaults, loop order and results.
 *
 * Differences, all additive:
 *   - results that the reference returns in std::vectors arrive through
 *     caller-owned host buffers (static profiles) or callbacks (dynamic
 *     snapshots, depinning steps), so the ABI stays plain C;
 *   - static_sweep relaxes all pinning lengths in one persistent launch when
 *     the field is a B-spline field (the lines are independent), one after
 *     another otherwise;
 *   - dynamic_anneal runs the step loop device-resident between snapshots
 *     (qew_langevin_run with the anneal's per-step coefficients);
 *   - optional knobs: L-BFGS history size, an explicit timestep, solver
 *     precision, and a force bisection to f_c after the ramp.
 */
#ifndef QEW_RUNS_H
#define QEW_RUNS_H

#include "qew_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* -------------------------------------------------------------- static */
/* StaticConfig, qew_runs.h:48-61. pinning_lengths_over_xi points to
 * n_pinning_lengths ratios lambda_p/xi (the caller keeps the array). */
typedef struct {
    int model;                 /* QEW_MODEL_*; default arclength */
    double amplitude;          /* 1 */
    double xi;                 /* 0.1, must match the field's xi */
    double Lx, Ly;             /* 32, 1 */
    int nx, ny;                /* 4096, 512 */
    double driving_force;      /* 0 */
    const double *pinning_lengths_over_xi; /* {0.01, 0.1, 1, 10, 100} */
    int n_pinning_lengths;
    double ftol;               /* 1e-6 */
    int max_iter;              /* 5000 */
    /* additive */
    int lbfgs_m;               /* L-BFGS history (LbfgsParams default 8) */
} qew_static_config;

/* StaticProfile, qew_runs.h:63-68 (h in the caller's buffer). */
typedef struct {
    double pinning_length_over_xi;
    double line_tension;
    qew_lbfgs_result result;
} qew_static_profile;

void qew_static_config_default(qew_static_config *c);
/* static_sweep(c, noise), qew_runs.h:70-102: for each ratio lp,
 * Gamma = amplitude * lp^1.5, flat start h = Ly/2, preconditioned L-BFGS
 * with shift 0.5 (Lx/nx) amplitude / xi^2. profiles[k] and the relaxed line
 * h_out[k * nx .. k * nx + nx) describe ratio k. */
qew_status qew_static_sweep(qew_ctx *ctx, const qew_field *field,
                            const qew_static_config *c,
                            qew_static_profile *profiles, double *h_out);

/* ------------------------------------------------------------- dynamic */
/* DynamicConfig, qew_runs.h:107-122. */
typedef struct {
    int model;                      /* arclength */
    double amplitude;               /* 1 */
    double xi;                      /* 0.1 */
    double pinning_length_over_xi;  /* 0.1 */
    double driving_force;           /* 0 */
    double Lx, Ly;                  /* 2, 1 */
    int nx, ny;                     /* 2048, 1024 */
    uint64_t seed;                  /* 1; the noise stream uses seed + 1 */
    double tau;                     /* 1 */
    double tl_start, tl_end;        /* 0.01, 0.0001 */
    double total_time;              /* 1000 */
    /* additive */
    double dt;                      /* > 0: this timestep instead of the
                                       heuristic of qew_runs.h:139-142 */
    int precision;                  /* QEW_PREC_FP64 (default) or FP32_SPLIT */
} qew_dynamic_config;

/* DynamicResult without the snapshots (qew_runs.h:129-134). */
typedef struct {
    double dt;
    double total_time;
    double line_tension;
    long long steps;
    int snapshots;
} qew_dynamic_result;

/* Called for each snapshot (qew_runs.h:171-174) with the host copy of h,
 * valid during the call. */
typedef void (*qew_snapshot_fn)(void *user, double t, const double *h, int n);

void qew_dynamic_config_default(qew_dynamic_config *c);
/* dynamic_anneal(c, noise), qew_runs.h:136-177. */
qew_status qew_dynamic_anneal(qew_ctx *ctx, const qew_field *field,
                              const qew_dynamic_config *c,
                              qew_snapshot_fn on_snapshot, void *user,
                              qew_dynamic_result *res);

/* ----------------------------------------------------------- depinning */
/* DepinningConfig, qew_runs.h:182-194. */
typedef struct {
    int model;                      /* arclength */
    double amplitude;               /* 1 */
    double xi;                      /* 0.1 */
    double pinning_length_over_xi;  /* 5 */
    double Lx, Ly;                  /* 8, 1 */
    int nx, ny;                     /* 1024, 256 */
    double f_step, f_max;           /* 1, 40 */
    qew_rk_params rp;               /* the caller fills it (the executable
                                       derives defaults from Ly/ny) */
    /* additive */
    double bisect_rtol;             /* > 0: bisect f_c to this relative
                                       width after the ramp */
    int precision;                  /* QEW_PREC_FP64 (default) or FP32_SPLIT */
} qew_depinning_config;

/* DepinningStep, qew_runs.h:196-200. */
typedef struct {
    double f;
    qew_rk_result result;
} qew_depinning_step;

typedef struct {
    double line_tension;
    double f_c_upper_bound;  /* first unblocked force, else -1 */
    int steps;
    /* additive (bisect_rtol > 0 and a bracket found; else f_c = -1) */
    double f_c, f_c_lo, f_c_hi;
    int bisect_blocks;
} qew_depinning_result;

/* Called for each ramp step; h (host copy, valid during the call) is given
 * only when the step blocked, as the reference stores it (qew_runs.h:234-236),
 * else NULL. */
typedef void (*qew_depinning_fn)(void *user, const qew_depinning_step *st,
                                 const double *h, int n);

void qew_depinning_config_default(qew_depinning_config *c);
/* depinning_ramp(c, noise), qew_runs.h:208-243. */
qew_status qew_depinning_ramp(qew_ctx *ctx, const qew_field *field,
                              const qew_depinning_config *c,
                              qew_depinning_fn on_step, void *user,
                              qew_depinning_result *res);

#ifdef __cplusplus
}
#endif

#endif /* QEW_RUNS_H */
