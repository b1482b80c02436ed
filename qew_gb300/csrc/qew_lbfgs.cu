// qew_lbfgs.cu -- L-BFGS minimiser (lbfgs.h:94-287).
//
// Form PLAIN keeps the reference's structure on the GPU: every vector
// operation is its own kernel, every reduction is read back to the host
// (one device->host synchronisation each), the scalars and the history ring
// live on the host, and the preconditioner is a cuFFT D2Z / divide / Z2D as
// kokkos-fft does on a CUDA build. It is the drop-in comparator ("one line,
// one launch per operation"). The device-resident form is in
// qew_lbfgs_resident.cu.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "qew_internal.cuh"
#include "qew_lbfgs_internal.cuh"
#include "qew_model_kernels.cuh"
#include "qew_vec.cuh"

namespace {

constexpr int kBS = 256;
inline int nblk(int n) { return (n + kBS - 1) / kBS; }

__global__ void k_precond_eig(int nh, int n, double kappa_over_dx, double shift, double *eig) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nh) return;
    const double pi = 3.14159265358979323846;
    const double s = sin(pi * (double)k / (double)n);
    eig[k] = kappa_over_dx * 4 * s * s + shift;  // lbfgs.h:138-143
}

// qhat_k /= eig_k (lbfgs.h:176-178), folding in kokkos-fft's backward 1/n.
__global__ void k_precond_divide(int nh, const double *__restrict__ eig, double inv_n,
                                 cufftDoubleComplex *qhat) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nh) return;
    const double e = eig[k];
    cufftDoubleComplex c = qhat[k];
    c.x = c.x / e * inv_n;
    c.y = c.y / e * inv_n;
    qhat[k] = c;
}

struct PlainFft {
    cufftHandle fwd = 0, inv = 0;
    bool have_fwd = false, have_inv = false;
    ~PlainFft() {
        if (have_fwd) cufftDestroy(fwd);
        if (have_inv) cufftDestroy(inv);
    }
    qew_status init(qew_ctx *ctx, int n) {
        if (cufftPlan1d(&fwd, n, CUFFT_D2Z, 1) != CUFFT_SUCCESS)
            return qew_fail(ctx, QEW_ERR_CUDA, "cufftPlan1d D2Z(%d) failed", n);
        have_fwd = true;
        if (cufftPlan1d(&inv, n, CUFFT_Z2D, 1) != CUFFT_SUCCESS)
            return qew_fail(ctx, QEW_ERR_CUDA, "cufftPlan1d Z2D(%d) failed", n);
        have_inv = true;
        cufftSetStream(fwd, ctx->stream);
        cufftSetStream(inv, ctx->stream);
        return QEW_OK;
    }
    // d = irfft(rfft(q) / eig); q is preserved (copied into the work buffer).
    qew_status apply(qew_ctx *ctx, int n, const double *q, double *work, const double *eig,
                     cufftDoubleComplex *qhat, double *d) {
        const int nh = n / 2 + 1;
        QEW_CUDA(ctx, cudaMemcpyAsync(work, q, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        if (cufftExecD2Z(fwd, work, qhat) != CUFFT_SUCCESS)
            return qew_fail(ctx, QEW_ERR_CUDA, "cufftExecD2Z failed");
        k_precond_divide<<<nblk(nh), kBS, 0, ctx->stream>>>(nh, eig, 1.0 / (double)n, qhat);
        QEW_TRY(qew_launch_check(ctx, "precond_divide"));
        if (cufftExecZ2D(inv, qhat, d) != CUFFT_SUCCESS)
            return qew_fail(ctx, QEW_ERR_CUDA, "cufftExecZ2D failed");
        ctx->launches += 2;  // the two cuFFT executions (library kernels)
        return QEW_OK;
    }
};

}  // namespace

double qew_precond_shift_rule(int n, double kappa, double physical_size, double shift) {
    if (shift <= 0) {  // lbfgs.h:131-135
        const double pi = 3.14159265358979323846;
        const double dx = physical_size / (double)n;
        const double s1 = std::sin(pi / (double)n);
        shift = (kappa / dx) * 4 * s1 * s1;
    }
    return shift;
}

qew_status qew_lbfgs_plain(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                           const qew_params *p, const qew_lbfgs_params *lp,
                           qew_lbfgs_result *res) {
    const int m = lp->m;
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    const int nh = n / 2 + 1;
    const size_t nhpad = ((size_t)nh + 31) & ~size_t(31);
    // g, g_new, d, q, s_tmp, y_tmp, fft work, S[m], Y[m], eig, qhat (complex)
    const size_t ndbl = npad * (7 + 2 * (size_t)std::max(m, 0)) + nhpad * 3;
    QEW_TRY(qew_scratch_reserve(ctx, ndbl * sizeof(double)));
    QEW_CUDA(ctx, cudaMemsetAsync(ctx->scratch, 0, ndbl * sizeof(double), ctx->stream));
    double *base = (double *)ctx->scratch;
    double *g = base, *g_new = base + npad, *d = base + 2 * npad, *q = base + 3 * npad;
    double *s_tmp = base + 4 * npad, *y_tmp = base + 5 * npad, *work = base + 6 * npad;
    std::vector<double *> S(m), Y(m);
    for (int k = 0; k < m; ++k) {
        S[k] = base + (7 + 2 * (size_t)k) * npad;
        Y[k] = base + (8 + 2 * (size_t)k) * npad;
    }
    double *eig = base + (7 + 2 * (size_t)m) * npad;
    cufftDoubleComplex *qhat = (cufftDoubleComplex *)(eig + nhpad);
    std::vector<double> rho(std::max(m, 1), 0.0), la(std::max(m, 1), 0.0);
    std::vector<int> slots;
    double gamma = 1.0;

    PlainFft fft;
    if (lp->precondition) {
        QEW_TRY(fft.init(ctx, n));
        const double dx = p->physical_size / (double)n;
        const double shift = qew_precond_shift_rule(n, p->line_tension, p->physical_size,
                                                    lp->precond_shift);
        k_precond_eig<<<nblk(nh), kBS, 0, ctx->stream>>>(nh, n, p->line_tension / dx, shift, eig);
        QEW_TRY(qew_launch_check(ctx, "precond_eig"));
    }

    auto dot = [&](const double *a, const double *b, double &out) -> qew_status {
        return vec_reduce<DotF, 1, false>(ctx, n, DotF{a, b}, &out);
    };
    auto max_abs = [&](const double *a, double &out) -> qew_status {
        return vec_reduce<AbsF, 1, true>(ctx, n, AbsF{a}, &out);
    };
    auto axpy = [&](double c, const double *x, double *y) -> qew_status {
        k_axpy<<<nblk(n), kBS, 0, ctx->stream>>>(n, c, x, y);
        return qew_launch_check(ctx, "axpy");
    };

    *res = qew_lbfgs_result{};
    QEW_TRY(qew_gradient_enqueue(ctx, field, d_h, n, p, QEW_PREC_FP64, g));
    int ls_fail_streak = 0;
    double phi = 0;
    for (int it = 0; it < lp->max_iter; ++it) {
        double gmax;
        QEW_TRY(max_abs(g, gmax));
        if (gmax < lp->ftol) {
            res->iterations = it;
            res->max_force = gmax;
            res->converged = 1;
            return QEW_OK;
        }
        QEW_CUDA(ctx, cudaMemcpyAsync(q, g, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        const int hs = (int)slots.size();
        for (int idx = hs - 1; idx >= 0; --idx) {
            const int row = slots[idx];
            double sq;
            QEW_TRY(dot(S[row], q, sq));
            const double a = rho[row] * sq;
            la[idx] = a;
            QEW_TRY(axpy(-a, Y[row], q));
        }
        if (lp->precondition) {
            QEW_TRY(fft.apply(ctx, n, q, work, eig, qhat, d));
        } else {
            const double g0 = slots.empty() ? 1.0 : gamma;
            k_scale<<<nblk(n), kBS, 0, ctx->stream>>>(n, g0, q, d);
            QEW_TRY(qew_launch_check(ctx, "scale"));
        }
        for (int idx = 0; idx < hs; ++idx) {
            const int row = slots[idx];
            double yd;
            QEW_TRY(dot(Y[row], d, yd));
            const double b = rho[row] * yd;
            QEW_TRY(axpy(la[idx] - b, S[row], d));
        }
        k_neg<<<nblk(n), kBS, 0, ctx->stream>>>(n, d);
        QEW_TRY(qew_launch_check(ctx, "neg"));

        double dphi0;
        QEW_TRY(dot(g, d, dphi0));
        if (dphi0 >= 0) {  // lbfgs.h:195-200
            slots.clear();
            k_neg_copy<<<nblk(n), kBS, 0, ctx->stream>>>(n, g, d);
            QEW_TRY(qew_launch_check(ctx, "sd"));
            double gg;
            QEW_TRY(dot(g, g, gg));
            dphi0 = -gg;
        }
        if (it == 0) {
            QEW_TRY(qew_objective(ctx, field, d_h, n, p, &phi));
            ++res->n_func_evals;
        }
        const double phi0 = phi;
        double alpha = 1.0;
        if (!lp->precondition && slots.empty()) {
            double gg;
            QEW_TRY(dot(g, g, gg));
            alpha = 1.0 / std::max(1.0, std::sqrt(gg));
        }
        bool ok = false, have_gn = false;
        for (int ls = 0; ls < lp->max_ls; ++ls) {
            double phi_trial;
            QEW_TRY(qew_objective_trial(ctx, field, d_h, d, alpha, n, p, &phi_trial));
            ++res->n_func_evals;
            if (phi_trial <= phi0 + lp->c1 * alpha * dphi0) {
                phi = phi_trial;
                ok = true;
                break;
            }
            if (lp->ls_fallback) {  // approximate-Wolfe slope test at q = h + alpha d
                QEW_CUDA(ctx, cudaMemcpyAsync(q, d_h, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                              ctx->stream));
                QEW_TRY(axpy(alpha, d, q));
                QEW_TRY(qew_gradient_enqueue(ctx, field, q, n, p, QEW_PREC_FP64, g_new));
                double dphia;
                QEW_TRY(dot(g_new, d, dphia));
                ++res->n_func_evals;
                if (dphia >= 0.9 * dphi0 && dphia <= (2.0 * 0.1 - 1.0) * dphi0 &&
                    phi_trial <= phi0 + 1e-10 * std::fabs(phi0)) {
                    phi = phi_trial;
                    ok = true;
                    have_gn = true;
                    break;
                }
            }
            alpha *= lp->ls_shrink;
        }
        if (!ok) {
            if (slots.empty() || ++ls_fail_streak > 2) {
                res->iterations = it;
                res->max_force = gmax;
                res->converged = 0;
                return QEW_OK;
            }
            slots.clear();
            ++res->n_ls_restarts;
            continue;
        }
        ls_fail_streak = 0;
        QEW_TRY(axpy(alpha, d, d_h));  // lbfgs_step, lbfgs.h:243-244
        if (!have_gn) QEW_TRY(qew_gradient_enqueue(ctx, field, d_h, n, p, QEW_PREC_FP64, g_new));
        double syy[3];
        QEW_TRY((vec_reduce<SyF, 3, false>(ctx, n, SyF{d, g_new, g, s_tmp, y_tmp, alpha}, syy)));
        const double sy = syy[0], ss = syy[1], yy = syy[2];
        if (sy > lp->curvature_eps * std::sqrt(ss * yy)) {
            int row;
            if ((int)slots.size() < m) {
                row = (int)slots.size();
            } else {
                row = slots.front();
                slots.erase(slots.begin());
            }
            std::swap(S[row], s_tmp);
            std::swap(Y[row], y_tmp);
            rho[row] = 1.0 / sy;
            gamma = sy / yy;
            slots.push_back(row);
        } else {
            ++res->n_curvature_skips;
        }
        std::swap(g, g_new);
    }
    res->iterations = lp->max_iter;
    double gm;
    QEW_TRY(max_abs(g, gm));
    res->max_force = gm;
    res->converged = 0;
    return QEW_OK;
}

qew_status qew_precond_plain(qew_ctx *ctx, const double *d_q, int n, double kappa,
                             double physical_size, double shift, double *d_out) {
    const int nh = n / 2 + 1;
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    const size_t nhpad = ((size_t)nh + 31) & ~size_t(31);
    QEW_TRY(qew_scratch_reserve(ctx, (npad + 3 * nhpad) * sizeof(double)));
    double *work = (double *)ctx->scratch;
    double *eig = work + npad;
    cufftDoubleComplex *qhat = (cufftDoubleComplex *)(eig + nhpad);
    PlainFft fft;
    QEW_TRY(fft.init(ctx, n));
    const double dx = physical_size / (double)n;
    const double sh = qew_precond_shift_rule(n, kappa, physical_size, shift);
    k_precond_eig<<<nblk(nh), kBS, 0, ctx->stream>>>(nh, n, kappa / dx, sh, eig);
    QEW_TRY(qew_launch_check(ctx, "precond_eig"));
    QEW_TRY(fft.apply(ctx, n, d_q, work, eig, qhat, d_out));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

extern "C" {

qew_status qew_lbfgs_default_params(qew_lbfgs_params *lp) {
    if (!lp) return QEW_ERR_INVALID;
    lp->m = 8;  // lbfgs.h:32-52
    lp->ftol = 1e-6;
    lp->max_iter = 10000;
    lp->c1 = 1e-4;
    lp->ls_shrink = 0.5;
    lp->max_ls = 30;
    lp->curvature_eps = 1e-12;
    lp->precondition = 0;
    lp->precond_shift = 0;
    lp->ls_fallback = 0;
    return QEW_OK;
}

qew_status qew_lbfgs_minimize_form(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                   const qew_params *p, const qew_lbfgs_params *lp, int form,
                                   qew_lbfgs_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !p || !lp || !res || n < 1 || lp->max_ls < 0 || lp->max_iter < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "lbfgs_minimize: bad arguments");
    // The reference indexes an empty history when m == 0 (lbfgs.h:264-268).
    if (lp->m < 1) return qew_fail(ctx, QEW_ERR_INVALID, "lbfgs_minimize: history length m must be >= 1");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (form == QEW_LBFGS_PLAIN) return qew_lbfgs_plain(ctx, field, d_h, n, p, lp, res);
    if (form == QEW_LBFGS_RESIDENT) return qew_lbfgs_resident(ctx, field, d_h, n, p, lp, res);
    return qew_fail(ctx, QEW_ERR_INVALID, "lbfgs_minimize: unknown form %d", form);
}

qew_status qew_lbfgs_minimize(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                              const qew_params *p, const qew_lbfgs_params *lp,
                              qew_lbfgs_result *res) {
    return qew_lbfgs_minimize_form(ctx, field, d_h, n, p, lp, QEW_LBFGS_RESIDENT, res);
}

qew_status qew_precond_apply(qew_ctx *ctx, const double *d_q, int n, double line_tension,
                             double physical_size, double shift, int form, double *d_out) {
    QEW_RANGE();
    if (!ctx || !d_q || !d_out || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "precond_apply: bad arguments");
    if (form == QEW_LBFGS_PLAIN)
        return qew_precond_plain(ctx, d_q, n, line_tension, physical_size, shift, d_out);
    if (form == QEW_LBFGS_RESIDENT)
        return qew_precond_resident(ctx, d_q, n, line_tension, physical_size, shift, d_out);
    return qew_fail(ctx, QEW_ERR_INVALID, "precond_apply: unknown form %d", form);
}

}  // extern "C"
