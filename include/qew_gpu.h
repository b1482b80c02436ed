/*
 * qew_gpu.h -- C ABI of the GB300-native qEW hot path.
 *
 * Plain C: opaque handles, plain pointers and sizes, status codes; no C++ or
 * torch types. Each entry point names the reference interface it replaces
 * (IMTEK-Simulation/qEW, paths relative to its source tree).
 *
 * Conventions
 *  - Device pointers (d_*) are caller-owned allocations on the context's
 *    device; host pointers (h_*) are ordinary or pinned host memory.
 *  - Work is enqueued on the context's CUDA stream (default: the legacy
 *    default stream, so it orders with other work there). Functions that
 *    return a host value (a scalar, a result struct) synchronise that stream
 *    before returning; the pure device-to-device kernels (gradient, sample,
 *    Langevin step) return as soon as their work is enqueued, like a Kokkos
 *    parallel_for.
 *  - A context is not thread-safe; use one per host thread.
 *  - Errors come back as a qew_status; qew_last_error() has the message.
 *    Where the reference throws (rk_block on odd n) the ABI returns
 *    QEW_ERR_ODD_LENGTH instead.
 *  - Every device-side wait is bounded and reports QEW_ERR_TIMEOUT.
 */
#ifndef QEW_GPU_H
#define QEW_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    QEW_OK = 0,
    QEW_ERR_INVALID = 1,     /* bad argument (size, null pointer, kind) */
    QEW_ERR_ODD_LENGTH = 2,  /* rk_block on odd n (rosso_krauth.h:134-136) */
    QEW_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    QEW_ERR_NOMEM = 4,       /* device allocation failed */
    QEW_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    QEW_ERR_UNSUPPORTED = 6  /* valid request that this library does not handle */
} qew_status;

typedef struct qew_ctx qew_ctx;
typedef struct qew_field qew_field;
typedef struct qew_langevin qew_langevin;

/* Model, qew_model.h:20 */
enum { QEW_MODEL_LINEAR = 0, QEW_MODEL_ARCLENGTH = 1 };

/* Params, qew_model.h:22-27. dx = physical_size / n. */
typedef struct {
    double physical_size;
    double line_tension;
    double driving_force;
    int model;
} qew_params;

/* Field kinds. QEW_FIELD_BSPLINE is FilteredNoise / DeviceNoise
 * (filtered_noise.h:67-210). The analytic kinds are the Noise functors the
 * reference's own tests inject, so those known-answer tests run unchanged:
 *   ZERO       ZeroNoise                       (test_lbfgs.cpp:24-27)
 *   CONST      ConstNoise{v0=p0}               (test_qew_model.cpp:38-42)
 *   HARMONIC   HarmonicWell{k=p0, y0=p1}       (test_lbfgs.cpp:30-38)
 *   WASHBOARD  SinusoidNoise{A=p0, k=p1}       (test_rosso_krauth.cpp:24-31)
 *   SINCOS     AnalyticNoise{amp=p0,kx=p1,ky=p2} (test_qew_model.cpp:22-34) */
enum {
    QEW_FIELD_BSPLINE = 0,
    QEW_FIELD_ZERO = 1,
    QEW_FIELD_CONST = 2,
    QEW_FIELD_HARMONIC = 3,
    QEW_FIELD_WASHBOARD = 4,
    QEW_FIELD_SINCOS = 5
};

/* Storage flags for B-spline fields. FP32_EDGE (only together with FP32)
 * adds the coefficients filtered along x at the half-integer columns,
 * E[j][e] = sum_a w_a(1/2) c[j][(e - 1 + a) mod nx] (computed in FP64,
 * stored FP32): the x half of the tensor-product sum at the edge midpoints
 * of a line with one point per field column (the x weights there are the
 * constants w(1/2) = 1/48, 23/48, 23/48, 1/48). With it the split-form
 * gradient on such a line reads 4 values per edge instead of 16; every other
 * line and call ignores it. */
enum { QEW_STORE_FP64 = 1, QEW_STORE_FP32 = 2, QEW_STORE_FP32_EDGE = 4,
       QEW_STORE_FP64_POLY = 8 };
/* FP64_POLY (only together with FP64) adds, for the same lines (one point
 * per field column), the FP64 cell polynomials of the x-filtered field: for
 * column e and row cell j the cubic V(e + 1/2, (j + t) dy), t in [0, 1), as
 * four FP64 numbers {q0, q1, q2, v0} with dV/dy = q0 + t (q1 + t q2) and
 * V = v0 + dy t (q0 + t (q1/2 + t q2/3)), computed once in FP64 from the
 * prefiltered coefficients (4x the FP64 coefficient memory, 32 bytes per
 * cell). The FP64 gradient on such a line then reads one 32-byte cell per
 * edge and evaluates two FMAs instead of the 16-tap tensor sum. Results stay
 * within 1e-15 of the gradient scale of the reference's order; they are not
 * bitwise equal to it (QEW_PREC_FP64_REFERENCE keeps that order). */

/* Precision of the gather in the model kernels. FP64 is the drop-in (parity)
 * form: it uses the FP64_POLY store when the field holds it and the line has
 * one point per field column, else the reference's 16-tap sum.
 * FP64_REFERENCE always evaluates the reference's expressions in its order
 * with its roundings (the 16-tap sum of filtered_noise.h:159-176, true
 * divisions, no fused multiply-adds), whatever the field stores: the
 * reference's results bit for bit, at a higher FP64 cost. FP32_SPLIT gathers
 * an FP32 coefficient copy at a height split into an integer cell plus an
 * FP32 fraction, with FP32 weights and sums (no FP64 arithmetic); its error
 * against FP64 is about 1e-6 of the gradient scale. */
enum { QEW_PREC_FP64 = 0, QEW_PREC_FP32_SPLIT = 1, QEW_PREC_FP64_REFERENCE = 2 };

/* LbfgsParams, lbfgs.h:32-52 (same fields, same defaults), plus
 * ls_fallback (no reference counterpart; default 0 = the reference's Armijo
 * search alone): 1 adds the approximate-Wolfe slope test (Hager & Zhang,
 * 2005) when the Armijo energy test fails, which lets the solve reach
 * gradient tolerances near 1e-8 where energy differences are below the
 * rounding of the energy. */
typedef struct {
    int m;
    double ftol;
    int max_iter;
    double c1;
    double ls_shrink;
    int max_ls;
    double curvature_eps;
    int precondition;
    double precond_shift;
    int ls_fallback;
} qew_lbfgs_params;

/* LbfgsResult, lbfgs.h:54-61 */
typedef struct {
    int iterations;
    double max_force;
    int converged;
    long n_func_evals;
    long n_curvature_skips;
    long n_ls_restarts;
} qew_lbfgs_result;

/* RkParams, rosso_krauth.h:34-41 */
typedef struct {
    double dstep;
    double max_advance;
    double root_tol;
    double sweep_tol;
    double runaway;
    int max_sweeps;
} qew_rk_params;

/* RkResult, rosso_krauth.h:43-49 */
typedef struct {
    int blocked;
    int runaway;
    int sweeps;
    double total_advance;
    double mean_h;
} qew_rk_result;

/* L-BFGS solver forms. PLAIN is the reference's host-driven loop, one
 * kernel (and, for each reduction, one device->host read) per vector
 * operation, with a cuFFT preconditioner: the one-line-per-launch comparator.
 * RESIDENT runs the whole solve in one kernel, one CTA per line: device-side
 * two-loop, the preconditioner as the exact factorised periodic solve of the
 * same circulant (equal to rfft / divide / irfft up to rounding), Armijo
 * search and history ring. */
enum { QEW_LBFGS_PLAIN = 0, QEW_LBFGS_RESIDENT = 1 };

/* ---------------------------------------------------------------- context */
const char *qew_status_string(qew_status s);
qew_status qew_ctx_create(int device, qew_ctx **out);
qew_status qew_ctx_destroy(qew_ctx *ctx);
/* cuda_stream is a cudaStream_t (NULL = legacy default stream). */
qew_status qew_ctx_set_stream(qew_ctx *ctx, void *cuda_stream);
qew_status qew_ctx_synchronize(qew_ctx *ctx);
/* Limits of the grid barriers in this context's later persistent cooperative
 * launches (Langevin run, Rosso-Krauth sweeps; no reference counterpart): a
 * wait gives up after max_polls polls of about 64 ns (<= 0: the default
 * 2^26) and the launch returns QEW_ERR_TIMEOUT. skip_block >= 0 makes that
 * CTA leave at its first barrier without arriving, so the others' waits run
 * out: a fault for tests of the timeout path (-1: none). */
qew_status qew_ctx_set_barrier_limits(qew_ctx *ctx, long long max_polls,
                                      int skip_block);
const char *qew_last_error(const qew_ctx *ctx);
/* Number of this library's kernels launched through ctx so far. */
uint64_t qew_ctx_launch_count(const qew_ctx *ctx);

/* ------------------------------------------------------------------ field */
/* FilteredNoise(const real_t *field, nx, ny, Lx, Ly), filtered_noise.h:189 /
 * filtered_noise.cpp:84-90 + build_coefficients (filtered_noise.cpp:92-136).
 * h_field is the reference's host layout, row-major [nx][ny] (i*ny + j).
 * The periodic cubic B-spline prefilter runs on the device; coefficients are
 * stored x-fastest ([ny][nx]) in FP64 and/or FP32 per store_flags. */
qew_status qew_field_create_from_host(qew_ctx *ctx, const double *h_field,
                                      int nx, int ny, double Lx, double Ly,
                                      int store_flags, qew_field **out);
/* Same, from a field already on the device (d_field, layout [nx][ny]). */
qew_status qew_field_create_from_device(qew_ctx *ctx, const double *d_field,
                                        int nx, int ny, double Lx, double Ly,
                                        int store_flags, qew_field **out);
/* Synthetic field generated on the device (no reference counterpart; the
 * on-device replacement of the host generation in FilteredNoise's seeded
 * constructor, filtered_noise.cpp:25-82, for per-request fields): white noise
 * from the Philox stream of `seed`, a periodic Gaussian filter of standard
 * deviation xi_x_cells / xi_y_cells grid cells along each axis (the real-space
 * form of exp(-(2 pi xi f)^2 / 2)), scaled to population std `amplitude`
 * (mean left in, as filtered_noise.cpp:61-79), then prefiltered as above. */
qew_status qew_field_create_generated(qew_ctx *ctx, int nx, int ny, double Lx,
                                      double Ly, double amplitude,
                                      double xi_x_cells, double xi_y_cells,
                                      uint64_t seed, int store_flags,
                                      qew_field **out);
/* FilteredNoise(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed), the reference's
 * seeded constructor (filtered_noise.h:183-185, filtered_noise.cpp:25-82):
 * unit-modulus random phases from std::mt19937_64(seed) through
 * std::uniform_real_distribution(0, 2 pi), drawn in the reference's order and
 * zeroed outside the correlation ellipse (fx xi_x)^2 + (fy xi_y)^2 <= 1, an
 * inverse FFT2 with 1/(nx ny) normalisation (cuFFT on the device), the real
 * part scaled to population std `amplitude` (mean kept), then prefiltered as
 * qew_field_create_from_host. The phases are drawn on the host (the
 * generator is sequential); everything after runs on the device. */
qew_status qew_field_create_seeded(qew_ctx *ctx, int nx, int ny, double Lx,
                                   double Ly, double amplitude, double xi_x,
                                   double xi_y, uint64_t seed, int store_flags,
                                   qew_field **out);
/* Analytic potentials (see the kind enum). */
qew_status qew_field_create_analytic(qew_ctx *ctx, int kind, double p0,
                                     double p1, double p2, qew_field **out);
qew_status qew_field_destroy(qew_field *field);
/* Download the FP64 coefficients in the reference's host layout [nx][ny]. */
qew_status qew_field_get_coefficients(qew_ctx *ctx, const qew_field *field,
                                      double *h_coef);
/* DeviceNoise::sample at m points (filtered_noise.h:103-134); any of the
 * outputs may be NULL. */
qew_status qew_field_sample(qew_ctx *ctx, const qew_field *field,
                            const double *d_x, const double *d_y, int m,
                            double *d_v, double *d_dvdx, double *d_dvdy);

/* ------------------------------------------------------------------ model */
/* objective(h, p, noise), qew_model.h:102-109. Deterministic reduction. */
qew_status qew_objective(qew_ctx *ctx, const qew_field *field,
                         const double *d_h, int n, const qew_params *p,
                         double *h_out);
/* objective(x0, d, alpha, p, noise), qew_model.h:112-119. */
qew_status qew_objective_trial(qew_ctx *ctx, const qew_field *field,
                               const double *d_x0, const double *d_d,
                               double alpha, int n, const qew_params *p,
                               double *h_out);
/* gradient(h, p, noise, grad[, ws]), qew_model.h:149-201, fused into one
 * kernel (edge pass and per-site combine share one launch). */
qew_status qew_gradient(qew_ctx *ctx, const qew_field *field,
                        const double *d_h, int n, const qew_params *p,
                        double *d_grad);
/* gradient with the gather precision selectable (QEW_PREC_*):
 * QEW_PREC_FP64_REFERENCE gives the reference's gradient bit for bit (its
 * operations in its order, true divisions, no fused multiply-adds). */
qew_status qew_gradient_prec(qew_ctx *ctx, const qew_field *field,
                             const double *d_h, int n, const qew_params *p,
                             int precision, double *d_grad);
/* gradient() of `count` lines of n points on one field, stored contiguously
 * (line k at offset k*n of d_h and d_grad), FP64 in and out (no reference
 * counterpart: the batched form of qew_model.h:149-201). With the
 * FP64_POLY store on a line with one point per field column the whole batch
 * is one persistent launch; otherwise one launch per line. */
qew_status qew_gradient_batch(qew_ctx *ctx, const qew_field *field, int count,
                              const double *d_h, int n, const qew_params *p,
                              int precision, double *d_grad);
/* Host-buffer gradient: copies h_h to the device, runs the gradient and
 * copies the result back into h_grad, all on the context's stream; returns
 * after the copy back has completed. */
qew_status qew_gradient_host(qew_ctx *ctx, const qew_field *field,
                             const double *h_h, int n, const qew_params *p,
                             int precision, double *h_grad);
/* Gradients of `count` host lines (h_h and h_grad hold count * n doubles,
 * line k at k * n; pinned memory lets the copies run asynchronously) in one
 * call: uploads, gradients and downloads of consecutive lines overlap on
 * three streams. No reference counterpart (the reference computes one
 * device-resident line per gradient() call, qew_model.h:149-201). */
qew_status qew_gradient_host_batch(qew_ctx *ctx, const qew_field *field,
                                   int count, const double *h_h, int n,
                                   const qew_params *p, int precision,
                                   double *h_grad);

/* FP32 split-index form of the gather (the bandwidth form; no reference
 * counterpart). Heights are carried in field y-cells as an integer cell plus
 * an FP32 fraction, h = (cell + frac) * dy. qew_split_heights / join convert
 * from / to FP64 heights; qew_gradient_split is gradient() (qew_model.h:149-201)
 * on split heights with FP32 output. Needs a field stored with QEW_STORE_FP32.
 * When the field also holds QEW_STORE_FP32_EDGE and the line has one point
 * per field column (n == nx, physical_size == Lx), each edge reads the
 * x-filtered store: 4 values instead of 16 taps, one persistent launch. The
 * result stays within the same error bound; it is not bitwise equal to the
 * 16-tap form, whose x sum runs in a different order. */
qew_status qew_split_heights(qew_ctx *ctx, const qew_field *field,
                             const double *d_h, int n, int32_t *d_cell,
                             float *d_frac);
qew_status qew_join_heights(qew_ctx *ctx, const qew_field *field,
                            const int32_t *d_cell, const float *d_frac, int n,
                            double *d_h);
qew_status qew_gradient_split(qew_ctx *ctx, const qew_field *field,
                              const int32_t *d_cell, const float *d_frac,
                              int n, const qew_params *p, float *d_grad);
/* The same for `count` lines of n points on one field, stored contiguously
 * (line k at offset k*n of each array), in one launch. */
qew_status qew_gradient_split_batch(qew_ctx *ctx, const qew_field *field,
                                    int count, const int32_t *d_cell,
                                    const float *d_frac, int n,
                                    const qew_params *p, float *d_grad);

/* Line energy without device allocation. No counterpart in the reference:
 * an addition for callers that cannot call cudaMalloc where they need the
 * energy (cudaMalloc/cudaFree can synchronise the whole device, which a
 * latency-bound serving loop cannot afford; a process whose device memory is
 * fully reserved up front gets out-of-memory from any extra allocation).
 * Same energy as qew_objective (within rounding of the reduction order),
 * written to the device pointer d_out on cuda_stream (NULL = legacy default
 * stream); returns once the work is enqueued. Its reduction scratch is a
 * static device array of QEW_NOALLOC_MAX_N/256 partial sums (32 KB) that
 * every GPU loading this library holds until exit; lines longer than
 * QEW_NOALLOC_MAX_N edges return QEW_ERR_INVALID. The field's device must be
 * the current device. The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress) and keeps it for that device's
 * current context; make that first call before any stream capture. A call
 * after the context was destroyed and created again (cudaDeviceReset) sees a
 * new context and looks the address up again; fields do not survive such a
 * reset, so create them anew first. All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define QEW_NOALLOC_MAX_N 1048576
qew_status qew_objective_noalloc(const qew_field *field, const double *d_h,
                                 int n, const qew_params *p, double *d_out,
                                 void *cuda_stream);

/* ----------------------------------------------------------------- L-BFGS */
qew_status qew_lbfgs_default_params(qew_lbfgs_params *lp);
/* lbfgs_minimize(h, p, noise, lp), lbfgs.h:94-287; relaxes d_h in place. */
qew_status qew_lbfgs_minimize(qew_ctx *ctx, const qew_field *field,
                              double *d_h, int n, const qew_params *p,
                              const qew_lbfgs_params *lp,
                              qew_lbfgs_result *res);
/* Same with the solver form chosen explicitly (QEW_LBFGS_*). */
qew_status qew_lbfgs_minimize_form(qew_ctx *ctx, const qew_field *field,
                                   double *d_h, int n, const qew_params *p,
                                   const qew_lbfgs_params *lp, int form,
                                   qew_lbfgs_result *res);
/* The preconditioner alone, d = M^{-1} q (lbfgs.h:116-146, 173-180), with
 * the shift rule of lbfgs.h:131-135 (shift <= 0 selects the auto shift). */
qew_status qew_precond_apply(qew_ctx *ctx, const double *d_q, int n,
                             double line_tension, double physical_size,
                             double shift, int form, double *d_out);

/* ------------------------------------------------------------------- FIRE */
/* FireParams, fire.h:21-31 (same fields, same defaults; dt_max is required). */
typedef struct {
    double dt_max;
    double dt_init;     /* <= 0: 0.1 * dt_max */
    double ftol;
    int max_iter;
    int n_min;
    double f_inc;
    double f_dec;
    double alpha_start;
    double f_alpha;
} qew_fire_params;

/* FireResult, fire.h:33-37 */
typedef struct {
    int iterations;
    double max_force;
    int converged;
} qew_fire_result;

qew_status qew_fire_default_params(qew_fire_params *fp);
/* fire_minimize(h, p, noise, fp), fire.h:41-131; relaxes d_h in place (one
 * kernel, one CTA). */
qew_status qew_fire_minimize(qew_ctx *ctx, const qew_field *field, double *d_h,
                             int n, const qew_params *p,
                             const qew_fire_params *fp, qew_fire_result *res);

/* ------------------------------------------------------------- statistics */
/* Roughness statistics of `count` periodic lines of n points (line k at
 * d_h + k * n, physical length L), the datasets the reference's
 * post-processing adds beside each profile (tools/postprocess_static.py:38-46:
 * ell, acf, q, psd). Its routines live in an external package that is not in
 * the reference tree, so the definitions are this project's, stated here:
 *   dx = L / n,  H_k = sum_i h_i exp(-2 pi i i k / n),  k = 0 .. n/2
 *   ell_k = k dx,  acf_k = (1/n) sum_i (h_{(i+k) mod n} - h_i)^2
 *   q_k = 2 pi k / L,  psd_k = (dx / n) |H_k|^2
 * Outputs (device): d_ell[n/2+1], d_acf[count][n/2+1], d_q[n/2+1],
 * d_psd[count][n/2+1]; any of d_ell, d_q and one of d_acf / d_psd may be
 * NULL. Transforms by cuFFT, batched over the lines. */
qew_status qew_line_statistics(qew_ctx *ctx, int count, const double *d_h, int n,
                               double physical_size, double *d_ell,
                               double *d_acf, double *d_q, double *d_psd);
/* The same from and to host arrays (h_h: count * n doubles). */
qew_status qew_line_statistics_host(qew_ctx *ctx, int count, const double *h_h,
                                    int n, double physical_size, double *h_ell,
                                    double *h_acf, double *h_q, double *h_psd);

/* --------------------------------------------------------------- ensemble */
/* Batched statics (no reference counterpart: the reference relaxes one line
 * per lbfgs_minimize call, lbfgs.h:94-96). One entry per independent line. */
typedef struct {
    const qew_field *field;  /* B-spline field: FP64 coefficients, and FP32
                                ones when the FP32 phase is used */
    double *d_h;             /* n heights on the device, relaxed in place */
    int n;
    qew_params p;
    double precond_shift;    /* per-line preconditioner shift (<= 0: auto) */
} qew_ensemble_line;

typedef struct {
    qew_lbfgs_params lbfgs;  /* m, final FP64 ftol, limits, line search */
    double ftol_fp32;        /* > 0: first relax on the FP32 split gather to
                                max|g| < ftol_fp32, then refine in FP64 */
    int max_iter_fp32;       /* iteration cap of that phase (<= 0: max_iter) */
} qew_ensemble_params;

/* Relaxes every line; results[k] describes line k (iterations and
 * evaluations of both phases summed, max_force/converged of the FP64
 * refinement). One persistent launch, longest lines first. */
qew_status qew_ensemble_minimize(qew_ctx *ctx, int count,
                                 const qew_ensemble_line *lines,
                                 const qew_ensemble_params *ep,
                                 qew_lbfgs_result *results);

/* ---------------------------------------------------------------- serving */
/* Continuous-batching server (no reference counterpart: the reference runs
 * one simulation per process, via its three executables). Requests wait in a
 * FIFO queue; `max_inflight` workers, each on its own CUDA stream, admit the
 * queue head as soon as its device-memory estimate fits in the HBM budget
 * left by the requests in flight, so new requests start while others run and
 * their kernels overlap. Each request generates its own field on the device
 * (qew_field_create_generated: n columns x rows rows, correlation xi cells,
 * unit variance, `seed`) and keeps all state device-resident. Results depend
 * only on the request: the same alone and in the mix. */
typedef struct qew_server qew_server;
enum { QEW_REQ_STATIC = 0, QEW_REQ_LANGEVIN = 1, QEW_REQ_DEPINNING = 2 };
typedef struct {
    int kind;              /* QEW_REQ_* */
    int n;                 /* line points = field columns, grid spacing 1 */
    int rows;              /* field rows */
    double xi;             /* field correlation length, cells */
    uint64_t seed;         /* field seed (Langevin increments: seed + 1) */
    int model;             /* QEW_MODEL_* (depinning: linear) */
    double line_tension;
    double driving_force;  /* static and Langevin */
    double ftol;           /* static: FP64 max|g| target (FP32 phase to 2e-5,
                              then FP64 refinement, preconditioned, m = 10) */
    int steps;             /* Langevin: steps at constant temperature */
    double temperature;    /* Langevin: kT; drift = dt, diff = sqrt(2 T dt) */
    double dt;
    double f_step, f_max;  /* depinning: force ramp (qew_runs.h:224-241) */
    double bisect_rtol;    /* depinning: f_c bisection tolerance */
    int max_sweeps;        /* depinning: RkParams::max_sweeps */
    double max_advance;    /* depinning: march cap per sweep, cells (<= 0: rows) */
    double runaway;        /* depinning: runaway mean advance, cells (<= 0: 2 rows) */
    double *h_out;         /* optional host buffer (n doubles) for the line */
} qew_request;
typedef struct {
    uint64_t id;
    int kind;
    qew_status status;
    double t_submit, t_start, t_end;  /* seconds on the server clock */
    int iterations;  /* static: L-BFGS iterations; Langevin: steps;
                        depinning: rk_block calls */
    double value;    /* static: energy; Langevin: mean height; depinning: f_c
                        (-1 if the ramp found no unblocked force) */
    double max_force;/* static: final max|g| */
    int converged;
} qew_response;
qew_status qew_server_create(int device, double hbm_budget_bytes,
                             int max_inflight, qew_server **out);
/* QEW_ERR_NOMEM if the request could never fit the budget. */
qew_status qew_server_submit(qew_server *s, const qew_request *req,
                             uint64_t *id);
/* Moves up to `max` finished responses into out; returns how many. */
int qew_server_poll(qew_server *s, qew_response *out, int max);
/* Waits until the queue is empty and nothing runs (QEW_ERR_TIMEOUT). */
qew_status qew_server_drain(qew_server *s, double timeout_s);
double qew_server_clock(const qew_server *s);
/* The device-resident loop for static requests (no reference counterpart):
 * static requests on lines of at most the lane limit (2048 points unless
 * qew_server_set_lane_limit changes it) at ftol 1e-8 are not
 * given to a worker; a persistent grid (one CTA per SM) takes them from a
 * ring in mapped host memory as the host publishes them and relaxes each on
 * one CTA (FP32 phase, FP64 refinement, the ensemble's arithmetic), so they
 * join running work without a launch of their own. A CTA without work for
 * about 16 ms leaves; the server relaunches the grid when jobs wait. Longer
 * lines take a thread-block cluster through a worker. *served: requests the
 * loop has finished; *launches: launches of its grid. QEW_ERR_UNSUPPORTED
 * when the loop could not be set up (all requests then go to workers). */
qew_status qew_server_lane_stats(qew_server *s, uint64_t *served,
                                 uint64_t *launches);
/* The lane limit: static requests on lines of at most max_n points (0: none,
 * at most QEW_LANE_CAP_N) go to the device-resident loop from the next
 * submission on. One CTA per line gives a long line alone a later result
 * than a thread-block cluster, and many lines together more solves/s. */
#define QEW_LANE_CAP_N 16384
qew_status qew_server_set_lane_limit(qew_server *s, int max_n);
qew_status qew_server_destroy(qew_server *s);

/* --------------------------------------------------------------- Langevin */
/* LangevinDynamics(n, seed), dynamics.h:31-32. Increments are N(0,1) from a
 * Philox4x32-10 counter stream keyed by seed, counter (site pair, step). */
qew_status qew_langevin_create(qew_ctx *ctx, int n, uint64_t seed,
                               qew_langevin **out);
qew_status qew_langevin_destroy(qew_langevin *lgv);
/* LangevinDynamics::step(h, p, noise, drift, diff), dynamics.h:34-64:
 * h_i += -drift * dE/dh_i + diff * xi_i (xi only when diff > 0). */
qew_status qew_langevin_step(qew_langevin *lgv, const qew_field *field,
                             double *d_h, const qew_params *p, double drift,
                             double diff);
/* Same step with caller-supplied increments d_xi[n] (trajectory parity). */
qew_status qew_langevin_step_increments(qew_langevin *lgv,
                                        const qew_field *field, double *d_h,
                                        const qew_params *p, double drift,
                                        double diff, const double *d_xi);
/* `steps` consecutive LangevinDynamics::step calls with per-step
 * coefficients h_drift[k], h_diff[k] (host arrays): the anneal loop of
 * dynamic_anneal (qew_runs.h:162-175) run in one cooperative persistent
 * kernel, same increments as the step-by-step calls (the Philox step
 * counter advances on each diff > 0 step). precision QEW_PREC_FP32_SPLIT
 * gathers the FP32 coefficients and draws the normals with an FP32
 * Box-Muller from the same Philox blocks; heights stay FP64. */
qew_status qew_langevin_run(qew_langevin *lgv, const qew_field *field,
                            double *d_h, const qew_params *p, int steps,
                            const double *h_drift, const double *h_diff,
                            int precision);
/* The increments the next qew_langevin_step would use, without stepping. */
qew_status qew_langevin_peek_increments(qew_langevin *lgv, double *d_xi);
/* Steps taken so far (the Philox step counter). */
uint64_t qew_langevin_steps(const qew_langevin *lgv);

/* ---------------------------------------------------------- Rosso-Krauth */
/* rk_site_velocity (rosso_krauth.h:51-82) of every site of d_h. */
qew_status qew_rk_site_velocity(qew_ctx *ctx, const qew_field *field,
                                const double *d_h, int n, const qew_params *p,
                                double *d_vel);
/* rk_block(h, p, noise, rp), rosso_krauth.h:128-194; advances d_h in place.
 * Odd n returns QEW_ERR_ODD_LENGTH (the reference throws). */
qew_status qew_rk_block(qew_ctx *ctx, const qew_field *field, double *d_h,
                        int n, const qew_params *p, const qew_rk_params *rp,
                        qew_rk_result *res);
/* rk_block forms: RESIDENT (the default of qew_rk_block) runs every sweep in
 * one cooperative persistent kernel with device-side verdicts; PLAIN keeps
 * the reference's host-driven loop (two colour kernels and one reduction
 * read back per sweep). Both give bit-identical lines. */
enum { QEW_RK_PLAIN = 0, QEW_RK_RESIDENT = 1 };
/* rk_block with the form and the gather precision chosen: QEW_PREC_FP32_SPLIT
 * (resident form only) evaluates site velocities on the FP32 coefficients
 * while heights, the no-passing update and the verdicts stay FP64;
 * QEW_PREC_FP64_REFERENCE evaluates them with the reference's arithmetic bit
 * for bit (both forms). */
qew_status qew_rk_block_form(qew_ctx *ctx, const qew_field *field,
                             double *d_h, int n, const qew_params *p,
                             const qew_rk_params *rp, int form, int precision,
                             qew_rk_result *res);
/* Force bisection for f_c (no reference counterpart; the reference ramps,
 * qew_runs.h:226-241): from a blocked d_h at f_lo and an unblocked f_hi,
 * bisect f, restarting each rk_block from the last blocked configuration,
 * until (f_hi - f_lo) <= rtol * f_hi. d_h ends as the blocked configuration
 * at f_lo; *f_c = (f_lo + f_hi) / 2. */
qew_status qew_depinning_bisect(qew_ctx *ctx, const qew_field *field,
                                double *d_h, int n, const qew_params *p,
                                const qew_rk_params *rp, double f_lo,
                                double f_hi, double rtol, int max_steps,
                                double *f_c, double *f_lo_out,
                                double *f_hi_out, int *n_blocks);
/* The same bisection with the velocity precision chosen (QEW_PREC_*). */
qew_status qew_depinning_bisect_prec(qew_ctx *ctx, const qew_field *field,
                                     double *d_h, int n, const qew_params *p,
                                     const qew_rk_params *rp, double f_lo,
                                     double f_hi, double rtol, int max_steps,
                                     int precision, double *f_c,
                                     double *f_lo_out, double *f_hi_out,
                                     int *n_blocks);
/* Outcome of a force bisection. Verdict of a block: 0 blocked, 1 runaway,
 * 2 neither (max_sweeps reached; counted as not blocked, as the reference's
 * ramp counts it, rosso_krauth.h:189-192, qew_runs.h:236-240). */
typedef struct {
    double f_c, f_lo, f_hi;
    int blocks;        /* rk_block calls */
    int n_blocked, n_runaway, n_timeout;
    int f_hi_verdict;  /* verdict that set f_hi last: 1 runaway, 2 max_sweeps
                          (f_c then depends on max_sweeps); 0: f_hi is the
                          caller's bracket end */
    long sweeps;       /* sweeps of all blocks */
} qew_bisect_result;
/* qew_depinning_bisect_prec reporting every block's verdict: h_verdicts (NULL
 * or max_steps ints) receives them in order. precision QEW_PREC_FP64_REFERENCE
 * evaluates the velocities with the reference's arithmetic bit for bit (true
 * divisions, no fused multiply-adds), so the verdicts, f_c and the critical
 * configuration are those of the reference's own evaluation order. */
qew_status qew_depinning_bisect_ex(qew_ctx *ctx, const qew_field *field,
                                   double *d_h, int n, const qew_params *p,
                                   const qew_rk_params *rp, double f_lo,
                                   double f_hi, double rtol, int max_steps,
                                   int precision, qew_bisect_result *res,
                                   int *h_verdicts);

/* ------------------------------------------------------------- autotuner */
/* Launch shapes chosen by measurement (no reference counterpart). Kernels
 * with several launch shapes that give bitwise-identical results time every
 * candidate on the first call of a (device, kernel, shape class) -- the
 * call's own work, CUDA events on the context's stream -- and keep the
 * fastest for the rest of the process:
 *   0 QEW_TUNE_GRADIENT_POLY   FP64 store gather: sites per thread {1,2,4} x
 *                              resident CTAs per SM {2,3,4} (9 candidates)
 *   1 QEW_TUNE_GRADIENT_SPLIT  FP32 split gather on the x-filtered store: sites
 *                              per thread {1,2} x CTAs per SM {4,6,8} (6)
 *   2 QEW_TUNE_RK_SEARCH       Rosso-Krauth forward-zero search: 8-lane groups,
 *                              lane pairs, one lane (3; timed for 8 sweeps on
 *                              a copy of the line advanced 24 sweeps; replaces
 *                              the warps-budget default only when more than
 *                              20 % faster)
 *   3 QEW_TUNE_LANGEVIN_RUN    qew_langevin_run: one grid barrier per step, or
 *                              K in {8,16,32} steps per barrier (temporal
 *                              blocking) at {1,2,4} CTAs per SM (10; timed for
 *                              64 steps of the run's schedule on a copy of the
 *                              line, on runs of at least 4096 steps)
 * The shape class is the log2 of the work (points) and the kernel's variant
 * (model; noise form and GPU share for the sweeps). */
enum { QEW_TUNE_GRADIENT_POLY = 0, QEW_TUNE_GRADIENT_SPLIT = 1, QEW_TUNE_RK_SEARCH = 2,
       QEW_TUNE_LANGEVIN_RUN = 3 };
/* on = 0: this context uses the hand-chosen default shapes. */
qew_status qew_ctx_set_autotune(qew_ctx *ctx, int on);
/* Fixes kernel's candidate for this context (-1: tuned or default again). */
qew_status qew_ctx_force_tune_candidate(qew_ctx *ctx, int kernel, int candidate);
/* The tuned choices of this process, one line per (device, kernel, class)
 * with every candidate's time; writes at most size-1 characters and a NUL,
 * returns the full length. */
int qew_tune_report(char *buf, int size);

/* ------------------------------------------------------- bounds checking */
/* The library built with -DQEW_BOUNDS_CHECK (qew_gb300/build.py, variant
 * "bounds_check", in _lib/bounds_check/) range-checks every field gather and
 * the gradient kernels' shared-memory indices on the device; an index
 * outside its array is clamped into range and recorded. No reference
 * counterpart (it stands in for a memory checker). Fills out[0] = the number
 * of out-of-range indices since the last report, out[1] = the first such
 * index, out[2] = its bound, out[3] = the source line of the check, after
 * synchronising the device, and clears them. QEW_ERR_UNSUPPORTED in the
 * normal build. */
qew_status qew_bounds_check_report(long long out[4]);

/* ------------------------------------------------------------ measurement */
/* FP64 FMA instructions per second of this GPU (no reference counterpart: the
 * roof of the FP64-pipe-bound gather). Eight resident CTAs per SM, each
 * thread `iters` rounds of eight independent FMA chains, timed with CUDA
 * events on the context's stream after one untimed launch; *ms_out (may be
 * NULL) is the timed launch's duration. */
qew_status qew_measure_fp64_fma_rate(qew_ctx *ctx, int iters, double *fma_per_s,
                                     double *ms_out);

#ifdef __cplusplus
}
#endif

#endif /* QEW_GPU_H */
