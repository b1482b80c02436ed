// qew_lbfgs_internal.cuh -- L-BFGS internals shared between solver forms.
#pragma once

#include "qew_internal.cuh"

// lbfgs.h:131-135: shift <= 0 selects the smallest non-zero elastic mode.
double qew_precond_shift_rule(int n, double kappa, double physical_size, double shift);

qew_status qew_lbfgs_plain(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                           const qew_params *p, const qew_lbfgs_params *lp,
                           qew_lbfgs_result *res);
qew_status qew_lbfgs_resident(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                              const qew_params *p, const qew_lbfgs_params *lp,
                              qew_lbfgs_result *res);
// Relaxes `count` lines of n points (d_h[k], parameters ps[k], preconditioner
// shift shifts[k]) on one field, one thread-block cluster per line; precision
// QEW_PREC_FP32_SPLIT gathers the field's FP32 coefficients. Returns
// QEW_ERR_UNSUPPORTED (recording nothing) when the lines are too short for a
// cluster or the device cannot run one; the caller then uses another form.
qew_status qew_lbfgs_cluster_lines(qew_ctx *ctx, const qew_field *field, int count,
                                   double *const *d_h, int n, const qew_params *ps,
                                   const double *shifts, const qew_lbfgs_params *lp,
                                   qew_lbfgs_result *res, int precision = QEW_PREC_FP64);
qew_status qew_precond_plain(qew_ctx *ctx, const double *d_q, int n, double kappa,
                             double physical_size, double shift, double *d_out);
qew_status qew_precond_resident(qew_ctx *ctx, const double *d_q, int n, double kappa,
                                double physical_size, double shift, double *d_out);

// Factorisation of the preconditioner M = a (2 - S - S^-1) + sigma, a = kappa/dx
// (the circulant whose eigenvalues are a 4 sin^2(pi k/n) + sigma, lbfgs.h:117-118):
// M = (a/z)(1 - zS)(1 - zS^-1) with z the root in (0,1) of
// z^2 - (2 + sigma/a) z + 1 = 0. Computed without cancellation from
// e = sigma/(2a): z - 1 = e - sqrt(e (2 + e)).
struct PrecondCoef {
    double z;       // pole
    double logz;    // log z
    double inv_1mzn;  // 1 / (1 - z^n)
    double gain;    // z / a  (so d = gain * w)
    double inv_sigma;  // used when a == 0 (M = sigma I)
    int scalar;     // 1 when a == 0
};
PrecondCoef qew_precond_coef(int n, double kappa, double physical_size, double shift);
