/*
 * qew_oracle.h -- CPU oracle for the qEW hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C, FP64 restatement of the reference algorithm, used by the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark as the
 * checker. It is never linked into, called by, or shipped with the CUDA
 * library; the product path has no CPU fallback.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the IMTEK-Simulation/qEW source tree). Arithmetic follows the reference
 * expression by expression and is compiled with -ffp-contract=off, so the
 * serial functions reproduce the reference's serial (Kokkos Serial) results.
 *
 * Field layout here is the reference's HOST layout: coef[i * ny + j], i the x
 * (column) index, j the y (row) index (filtered_noise.h:208,
 * filtered_noise.cpp:102-104).
 */
#ifndef QEW_ORACLE_H
#define QEW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Noise kinds: the production B-spline field and the analytic potentials the
 * reference's own tests inject through the Noise template parameter. */
enum {
    QO_NOISE_BSPLINE = 0,  /* DeviceNoise, filtered_noise.h:67-177 */
    QO_NOISE_ZERO = 1,     /* ZeroNoise, test_lbfgs.cpp:24-27 */
    QO_NOISE_CONST = 2,    /* ConstNoise{v0}, test_qew_model.cpp:38-42 */
    QO_NOISE_HARMONIC = 3, /* HarmonicWell{k, y0}, test_lbfgs.cpp:30-38 */
    QO_NOISE_WASHBOARD = 4,/* SinusoidNoise{A, k}, test_rosso_krauth.cpp:24-31 */
    QO_NOISE_SINCOS = 5    /* AnalyticNoise{amp, kx, ky}, test_qew_model.cpp:22-34 */
};

typedef struct {
    int kind;
    const double *coef; /* B-spline coefficients, coef[i*ny + j] */
    int nx, ny;
    double dx, dy;      /* field grid spacing Lx/nx, Ly/ny */
    double p0, p1, p2;  /* analytic parameters (see enum) */
} qo_noise;

typedef struct {
    double physical_size; /* Params, qew_model.h:22-27 */
    double line_tension;
    double driving_force;
    int model;            /* 0 Linear, 1 Arclength */
} qo_params;

typedef struct { /* LbfgsParams, lbfgs.h:32-52 */
    int m;
    double ftol;
    int max_iter;
    double c1;
    double ls_shrink;
    int max_ls;
    double curvature_eps;
    int precondition;
    double precond_shift;
    int ls_fallback; /* extension (not in the reference): approximate-Wolfe
                        slope test when the Armijo test fails */
} qo_lbfgs_params;

typedef struct { /* LbfgsResult, lbfgs.h:54-61 */
    int iterations;
    double max_force;
    int converged;
    long n_func_evals;
    long n_curvature_skips;
    long n_ls_restarts;
} qo_lbfgs_result;

typedef struct { /* RkParams, rosso_krauth.h:34-41 */
    double dstep, max_advance, root_tol, sweep_tol, runaway;
    int max_sweeps;
} qo_rk_params;

typedef struct { /* RkResult, rosso_krauth.h:43-49 */
    int blocked, runaway, sweeps;
    double total_advance, mean_h;
} qo_rk_result;

typedef struct { /* FireParams, fire.h:21-31 */
    double dt_max, dt_init, ftol;
    int max_iter, n_min;
    double f_inc, f_dec, alpha_start, f_alpha;
} qo_fire_params;

typedef struct { /* FireResult, fire.h:33-37 */
    int iterations;
    double max_force;
    int converged;
} qo_fire_result;

/* ---- B-spline field (filtered_noise.h / filtered_noise.cpp) ---- */
void qo_bspline_weights_value(double t, double w[4]);
void qo_bspline_weights(double t, double w[4], double dw[4]);
void qo_sample(const qo_noise *nz, double x, double y, double *v, double *dvdx,
               double *dvdy);
double qo_sample_value(const qo_noise *nz, double x, double y);
double qo_sample_dy(const qo_noise *nz, double x, double y);
void qo_sample_many(const qo_noise *nz, const double *x, const double *y, int m,
                    double *v, double *dvdx, double *dvdy);
/* Prefilter field (row-major i*ny+j) -> coef (same layout). */
int qo_prefilter(const double *field, int nx, int ny, double *coef);

/* ---- std::mt19937_64 and the seeded field (filtered_noise.cpp:25-82) ---- */
typedef struct { uint64_t mt[312]; int idx; } qo_mt64;
void qo_mt64_seed(qo_mt64 *g, uint64_t seed);
uint64_t qo_mt64_next(qo_mt64 *g);
double qo_mt64_uniform(qo_mt64 *g, double a, double b);
int qo_seeded_field(int nx, int ny, double Lx, double Ly, double amplitude, double xi_x,
                    double xi_y, uint64_t seed, double *field);

/* ---- complex / real FFT (kokkos-fft semantics: forward unnormalised,
 * backward 1/n) ---- */
int qo_fft(double *re, double *im, int n, int inverse);
int qo_rfft(const double *x, int n, double *re, double *im);   /* n/2+1 out */
int qo_irfft(const double *re, const double *im, int n, double *x);

/* ---- model (qew_model.h) ---- */
double qo_objective(const double *h, int n, const qo_params *p,
                    const qo_noise *nz);
double qo_objective_trial(const double *x0, const double *d, double alpha,
                          int n, const qo_params *p, const qo_noise *nz);
void qo_gradient(const double *h, int n, const qo_params *p,
                 const qo_noise *nz, double *grad);
/* fire_minimize, fire.h:41-131 (serial) */
void qo_fire_minimize(double *h, int n, const qo_params *p, const qo_noise *nz,
                      const qo_fire_params *fp, qo_fire_result *res);
/* Thread-parallel gradient/objective (OpenMP): the timed CPU baseline. */
void qo_gradient_omp(const double *h, int n, const qo_params *p,
                     const qo_noise *nz, double *grad);
double qo_objective_omp(const double *h, int n, const qo_params *p,
                        const qo_noise *nz);
int qo_omp_max_threads(void);

/* ---- L-BFGS (lbfgs.h) ---- */
void qo_lbfgs_default_params(qo_lbfgs_params *lp);
int qo_lbfgs_minimize(double *h, int n, const qo_params *p,
                      const qo_noise *nz, const qo_lbfgs_params *lp,
                      qo_lbfgs_result *res);
/* Preconditioner application d = M^{-1} q (lbfgs.h:116-146, 173-180). */
int qo_precond_apply(const double *q, int n, double kappa, double physical_size,
                     double shift, double *d);

/* ---- Langevin (dynamics.h) with caller-supplied N(0,1) increments ---- */
void qo_langevin_step(double *h, int n, const qo_params *p, const qo_noise *nz,
                      double drift, double diff, const double *xi,
                      double *grad_scratch);

/* ---- Rosso-Krauth (rosso_krauth.h) ---- */
double qo_rk_site_velocity(int i, int n, double dx, double lt, double f,
                           int model, double hi, double hl, double hr,
                           const qo_noise *nz);
double qo_rk_forward_zero(int i, int n, double dx, double lt, double f,
                          int model, double hi, double hl, double hr,
                          const qo_noise *nz, const qo_rk_params *rp,
                          int *found);
/* returns 0, or -1 for odd n (the reference throws std::invalid_argument) */
int qo_rk_block(double *h, int n, const qo_params *p, const qo_noise *nz,
                const qo_rk_params *rp, qo_rk_result *res);
/* Force bisection protocol for f_c: see qew_oracle.c. */
int qo_depinning_bisect(double *h, int n, const qo_params *p,
                        const qo_noise *nz, const qo_rk_params *rp,
                        double f_lo, double f_hi, double rtol, int max_steps,
                        double *f_c, double *f_lo_out, double *f_hi_out,
                        int *n_blocks);
int qo_depinning_bisect_ex(double *h, int n, const qo_params *p,
                           const qo_noise *nz, const qo_rk_params *rp,
                           double f_lo, double f_hi, double rtol, int max_steps,
                           double *f_c, double *f_lo_out, double *f_hi_out,
                           int *n_blocks, int *verdicts, long *sweeps);

/* ---- Philox4x32-10 counter RNG + Box-Muller normals (shared with the GPU
 * Langevin step, so the oracle can regenerate the same increments) ---- */
void qo_philox_normals(uint64_t seed, uint64_t step, int n, double *out);
void qo_langevin_step_philox(double *h, int n, const qo_params *p, const qo_noise *nz,
                             double drift, double diff, uint64_t seed, uint64_t step,
                             double *grad, double *xi, int par);
void qo_omp_set_threads(int k);

#ifdef __cplusplus
}
#endif

#endif /* QEW_ORACLE_H */
