// qew_runs.cu -- static_sweep, dynamic_anneal and depinning_ramp
// (qew_runs.h:45-243 of the reference) over this library's solvers.
//
// The drivers are host orchestration: the configuration semantics, loop
// order, Larkin map Gamma = amplitude * (lambda_p/xi)^1.5 (qew_runs.h:27-34),
// flat start at Ly/2 and the results are the reference's; the work inside
// each step runs on the GPU:
//   * static_sweep: the ratios are independent lines, relaxed together in one
//     launch -- a thread-block cluster per line for long lines, else the
//     ensemble kernel's CTA per line on a B-spline field (FP64 throughout) --
//     or one resident L-BFGS solve after another;
//   * dynamic_anneal: the per-step anneal coefficients are produced on the
//     host exactly as the reference's loop does, and the steps between two
//     snapshots run device-resident (qew_langevin_run);
//   * depinning_ramp: resident rk_block per force, restarting from the last
//     configuration; optionally a force bisection to f_c afterwards.
#include "qew_internal.cuh"
#include "qew_lbfgs_internal.cuh"
#include "qew_runs.h"

#include <cmath>
#include <vector>

namespace {

double larkin_tension(double lp_over_xi, double amplitude) {
    return std::pow(lp_over_xi, 1.5) * amplitude;  // qew_runs.h:77, 143-144, 210-211
}

const double kDefaultRatios[] = {0.01, 0.1, 1.0, 10.0, 100.0};

// Device line of n doubles, filled with v (the flat start).
struct DeviceLine {
    double *d = nullptr;
    qew_ctx *ctx = nullptr;
    ~DeviceLine() {
        if (d) {
            cudaStreamSynchronize(ctx->stream);
            qew_free_async(d, ctx->stream);
        }
    }
};

qew_status alloc_lines(qew_ctx *ctx, DeviceLine &L, size_t count) {
    L.ctx = ctx;
    return qew_alloc_async(ctx, (void **)&L.d, count * sizeof(double));
}

qew_status fill_flat(qew_ctx *ctx, double *d, size_t count, double v) {
    std::vector<double> h(count, v);
    QEW_CUDA(ctx, cudaMemcpyAsync(d, h.data(), count * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

qew_status to_host(qew_ctx *ctx, const double *d, int n, std::vector<double> &h) {
    h.resize(n);
    QEW_CUDA(ctx, cudaMemcpyAsync(h.data(), d, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

bool model_ok(int m) { return m == QEW_MODEL_LINEAR || m == QEW_MODEL_ARCLENGTH; }

}  // namespace

extern "C" {

void qew_static_config_default(qew_static_config *c) {
    if (!c) return;
    *c = qew_static_config{};
    c->model = QEW_MODEL_ARCLENGTH;
    c->amplitude = 1.0;
    c->xi = 0.1;
    c->Lx = 32.0;
    c->Ly = 1.0;
    c->nx = 4096;
    c->ny = 512;
    c->driving_force = 0.0;
    c->pinning_lengths_over_xi = kDefaultRatios;
    c->n_pinning_lengths = 5;
    c->ftol = 1e-6;
    c->max_iter = 5000;
    c->lbfgs_m = 8;
}

qew_status qew_static_sweep(qew_ctx *ctx, const qew_field *field, const qew_static_config *c,
                            qew_static_profile *profiles, double *h_out) {
    QEW_RANGE();
    if (!ctx || !field || !c || c->nx < 1 || c->n_pinning_lengths < 0 ||
        (c->n_pinning_lengths > 0 && (!c->pinning_lengths_over_xi || !profiles || !h_out)) ||
        !model_ok(c->model))
        return qew_fail(ctx, QEW_ERR_INVALID, "static_sweep: bad arguments");
    const int K = c->n_pinning_lengths, n = c->nx;
    if (K == 0) return QEW_OK;
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    qew_lbfgs_params lp;
    qew_lbfgs_default_params(&lp);
    lp.m = c->lbfgs_m > 0 ? c->lbfgs_m : lp.m;
    lp.ftol = c->ftol;
    lp.max_iter = c->max_iter;
    // Inverse-Laplacian preconditioner with the pinning-curvature shift
    // ~ dx A / xi^2 (qew_runs.h:87-91).
    lp.precondition = 1;
    lp.precond_shift = 0.5 * (c->Lx / c->nx) * c->amplitude / (c->xi * c->xi);

    DeviceLine lines;
    QEW_TRY(alloc_lines(ctx, lines, (size_t)K * n));
    QEW_TRY(fill_flat(ctx, lines.d, (size_t)K * n, 0.5 * c->Ly));  // flat start
    std::vector<qew_params> ps(K);
    for (int k = 0; k < K; ++k) {
        qew_params &p = ps[k];
        p.physical_size = c->Lx;
        p.line_tension = larkin_tension(c->pinning_lengths_over_xi[k], c->amplitude);
        p.driving_force = c->driving_force;
        p.model = c->model;
        profiles[k].pinning_length_over_xi = c->pinning_lengths_over_xi[k];
        profiles[k].line_tension = p.line_tension;
    }
    std::vector<qew_lbfgs_result> res(K);
    // long lines: one thread-block cluster per ratio; else the ensemble kernel
    // (one CTA per ratio) on a B-spline field, or one solve after another
    std::vector<double *> hp(K);
    std::vector<double> shifts(K, lp.precond_shift);
    for (int k = 0; k < K; ++k) hp[k] = lines.d + (size_t)k * n;
    const qew_status cs = qew_lbfgs_cluster_lines(ctx, field, K, hp.data(), n, ps.data(),
                                                  shifts.data(), &lp, res.data());
    if (cs != QEW_OK && cs != QEW_ERR_UNSUPPORTED) return cs;
    if (cs == QEW_ERR_UNSUPPORTED) {
        if (field->kind == QEW_FIELD_BSPLINE && field->coef64) {
            std::vector<qew_ensemble_line> el(K);
            for (int k = 0; k < K; ++k)
                el[k] = qew_ensemble_line{field, hp[k], n, ps[k], lp.precond_shift};
            qew_ensemble_params ep{};
            ep.lbfgs = lp;
            ep.ftol_fp32 = 0.0;  // FP64 throughout, as the reference
            QEW_TRY(qew_ensemble_minimize(ctx, K, el.data(), &ep, res.data()));
        } else {
            for (int k = 0; k < K; ++k)
                QEW_TRY(qew_lbfgs_minimize(ctx, field, hp[k], n, &ps[k], &lp, &res[k]));
        }
    }
    QEW_CUDA(ctx, cudaMemcpyAsync(h_out, lines.d, (size_t)K * n * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < K; ++k) profiles[k].result = res[k];
    return QEW_OK;
}

void qew_dynamic_config_default(qew_dynamic_config *c) {
    if (!c) return;
    *c = qew_dynamic_config{};
    c->model = QEW_MODEL_ARCLENGTH;
    c->amplitude = 1.0;
    c->xi = 0.1;
    c->pinning_length_over_xi = 0.1;
    c->driving_force = 0.0;
    c->Lx = 2.0;
    c->Ly = 1.0;
    c->nx = 2048;
    c->ny = 1024;
    c->seed = 1;
    c->tau = 1.0;
    c->tl_start = 0.01;
    c->tl_end = 0.0001;
    c->total_time = 1000.0;
    c->dt = 0.0;
    c->precision = QEW_PREC_FP64;
}

qew_status qew_dynamic_anneal(qew_ctx *ctx, const qew_field *field, const qew_dynamic_config *c,
                              qew_snapshot_fn on_snapshot, void *user, qew_dynamic_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !c || !res || c->nx < 1 || !model_ok(c->model) || !(c->tau > 0) ||
        !(c->amplitude != 0) || !std::isfinite(c->total_time))
        return qew_fail(ctx, QEW_ERR_INVALID, "dynamic_anneal: bad arguments");
    const double tau = c->tau;
    // qew_dynamic.py timestep heuristic (qew_runs.h:139-142).
    const double fac = c->xi / std::max(c->tl_start, c->tl_end);
    const double dt = c->dt > 0 ? c->dt : std::min(0.1, tau / 10 * std::min(fac, fac * fac));
    if (!(dt > 0) || !std::isfinite(dt))
        return qew_fail(ctx, QEW_ERR_INVALID, "dynamic_anneal: timestep %g", dt);
    if (c->total_time / dt > 1e12)
        return qew_fail(ctx, QEW_ERR_INVALID, "dynamic_anneal: %g steps", c->total_time / dt);
    const double line_tension = larkin_tension(c->pinning_length_over_xi, c->amplitude);
    qew_params p{};
    p.physical_size = c->Lx;
    p.line_tension = line_tension;
    p.driving_force = c->driving_force;
    p.model = c->model;
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));

    DeviceLine h;
    QEW_TRY(alloc_lines(ctx, h, (size_t)c->nx));
    QEW_TRY(fill_flat(ctx, h.d, (size_t)c->nx, 0.5 * c->Ly));  // flat start
    qew_langevin *dyn = nullptr;
    QEW_TRY(qew_langevin_create(ctx, c->nx, c->seed + 1, &dyn));
    struct Guard {
        qew_langevin *l;
        ~Guard() { qew_langevin_destroy(l); }
    } guard{dyn};

    res->dt = dt;
    res->total_time = c->total_time;
    res->line_tension = line_tension;
    res->steps = 0;
    res->snapshots = 0;

    // The reference's loop (qew_runs.h:161-175) evaluated on the host for its
    // coefficients; the steps themselves are batched into device-resident runs
    // that end at each snapshot or after kChunk steps.
    constexpr int kChunk = 1 << 16;
    std::vector<double> drift, diff, hh;
    drift.reserve(kChunk);
    diff.reserve(kChunk);
    auto flush = [&]() -> qew_status {
        if (drift.empty()) return QEW_OK;
        QEW_TRY(qew_langevin_run(dyn, field, h.d, &p, (int)drift.size(), drift.data(), diff.data(),
                                 c->precision));
        res->steps += (long long)drift.size();
        drift.clear();
        diff.clear();
        return QEW_OK;
    };
    double t = 0.0;
    double next_save = 10 * dt;
    double tl = c->tl_start;
    while (t < c->total_time) {
        drift.push_back(tl * dt / (tau * c->amplitude));
        diff.push_back(tl * std::sqrt(2 * dt / tau));
        tl = c->tl_start + (c->tl_end - c->tl_start) * (t / c->total_time);  // anneal
        t += dt;
        if (t > next_save - dt / 2) {
            QEW_TRY(flush());
            QEW_TRY(to_host(ctx, h.d, c->nx, hh));
            if (on_snapshot) on_snapshot(user, t, hh.data(), c->nx);
            ++res->snapshots;
            next_save *= 10;
        } else if ((int)drift.size() == kChunk) {
            QEW_TRY(flush());
        }
    }
    QEW_TRY(flush());
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

void qew_depinning_config_default(qew_depinning_config *c) {
    if (!c) return;
    *c = qew_depinning_config{};
    c->model = QEW_MODEL_ARCLENGTH;
    c->amplitude = 1.0;
    c->xi = 0.1;
    c->pinning_length_over_xi = 5.0;
    c->Lx = 8.0;
    c->Ly = 1.0;
    c->nx = 1024;
    c->ny = 256;
    c->f_step = 1.0;
    c->f_max = 40.0;
    // RkParams defaults, rosso_krauth.h:34-41
    c->rp.dstep = 0.0;
    c->rp.max_advance = 0.0;
    c->rp.root_tol = 1e-10;
    c->rp.sweep_tol = 1e-9;
    c->rp.runaway = 0.0;
    c->rp.max_sweeps = 200000;
    c->bisect_rtol = 0.0;
    c->precision = QEW_PREC_FP64;
}

qew_status qew_depinning_ramp(qew_ctx *ctx, const qew_field *field, const qew_depinning_config *c,
                              qew_depinning_fn on_step, void *user, qew_depinning_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !c || !res || c->nx < 1 || !model_ok(c->model) ||
        !std::isfinite(c->f_step) || !std::isfinite(c->f_max))
        return qew_fail(ctx, QEW_ERR_INVALID, "depinning_ramp: bad arguments");
    if (c->nx % 2) return qew_fail(ctx, QEW_ERR_ODD_LENGTH, "rk_block: n must be even");
    // The force loop k * f_step <= f_max (qew_runs.h:224-227) ends only for
    // f_step > 0 (or when it never starts, f_max < 0); bound its length.
    if (c->f_max >= 0 && !(c->f_step > 0))
        return qew_fail(ctx, QEW_ERR_INVALID, "depinning_ramp: need f_step > 0 (f_max >= 0)");
    if (c->f_step > 0 && c->f_max / c->f_step > 1e9)
        return qew_fail(ctx, QEW_ERR_INVALID, "depinning_ramp: more than 1e9 forces");
    const double line_tension = larkin_tension(c->pinning_length_over_xi, c->amplitude);
    qew_params p{};
    p.physical_size = c->Lx;
    p.line_tension = line_tension;
    p.model = c->model;
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));

    DeviceLine h, h_lo;
    QEW_TRY(alloc_lines(ctx, h, (size_t)c->nx));
    QEW_TRY(fill_flat(ctx, h.d, (size_t)c->nx, 0.5 * c->Ly));  // flat start
    const bool bisect = c->bisect_rtol > 0;
    if (bisect) QEW_TRY(alloc_lines(ctx, h_lo, (size_t)c->nx));

    res->line_tension = line_tension;
    res->f_c_upper_bound = -1;
    res->steps = 0;
    res->f_c = res->f_c_lo = res->f_c_hi = -1;
    res->bisect_blocks = 0;
    bool have_lo = false;
    double f_lo = 0;
    std::vector<double> hh;
    // Integer force counter, as qew_runs.h:224-227 (no drift of f).
    for (int k = 0; (double)k * c->f_step <= c->f_max; ++k) {
        const double f = (double)k * c->f_step;
        p.driving_force = f;
        qew_depinning_step st{};
        st.f = f;
        QEW_TRY(qew_rk_block_form(ctx, field, h.d, c->nx, &p, &c->rp, QEW_RK_RESIDENT,
                                  c->precision, &st.result));  // restart from previous
        ++res->steps;
        if (st.result.blocked) {
            QEW_TRY(to_host(ctx, h.d, c->nx, hh));
            if (bisect) {
                QEW_CUDA(ctx, cudaMemcpyAsync(h_lo.d, h.d, (size_t)c->nx * sizeof(double),
                                              cudaMemcpyDeviceToDevice, ctx->stream));
                have_lo = true;
                f_lo = f;
            }
            if (on_step) on_step(user, &st, hh.data(), c->nx);
        } else {
            res->f_c_upper_bound = f;  // the first unblocked force brackets f_c
            if (on_step) on_step(user, &st, nullptr, c->nx);
            break;
        }
    }
    if (bisect && have_lo && res->f_c_upper_bound >= 0) {
        p.driving_force = f_lo;
        QEW_TRY(qew_depinning_bisect_prec(ctx, field, h_lo.d, c->nx, &p, &c->rp, f_lo,
                                          res->f_c_upper_bound, c->bisect_rtol, 64, c->precision,
                                          &res->f_c, &res->f_c_lo, &res->f_c_hi,
                                          &res->bisect_blocks));
    }
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

}  // extern "C"
