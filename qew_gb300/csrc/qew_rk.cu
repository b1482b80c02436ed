// qew_rk.cu -- Rosso-Krauth red-black no-passing construction
// (rk_block, rosso_krauth.h:128-194) and the f_c bisection driver.
//
// rk_block runs its sweeps in a persistent kernel (qew_rk_resident.cu) when
// the line is on a B-spline field; the host-driven form below mirrors the
// reference's structure (two colour kernels and one reduction read back per
// sweep) and serves every field kind.
#include <cmath>
#include <vector>

#include "qew_internal.cuh"
#include "qew_rk_device.cuh"
#include "qew_rk_internal.cuh"
#include "qew_vec.cuh"

namespace {

constexpr int kBS = 256;

// One colour of one sweep (rosso_krauth.h:154-165): thread k owns site 2k+color.
template <class Noise>
__global__ void k_rk_colour(Noise nz, double *__restrict__ h, double *__restrict__ adv, int n,
                            double dx, double lt, double f, int model, int color, RkP rp) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 2 * k + color;
    if (i >= n) return;
    const int im = (i == 0) ? n - 1 : i - 1;
    const int ip = (i + 1 == n) ? 0 : i + 1;
    bool found = false;
    const double hi = h[i];
    const double hnew = rk_forward_zero(nz, i, n, dx, lt, f, model, hi, h[im], h[ip], rp, found);
    adv[i] = hnew - hi;
    h[i] = hnew;
}

template <class Noise>
__global__ void k_rk_velocity(Noise nz, const double *__restrict__ h, int n, double dx, double lt,
                              double f, int model, double *__restrict__ vel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int im = (i == 0) ? n - 1 : i - 1;
    const int ip = (i + 1 == n) ? 0 : i + 1;
    vel[i] = rk_site_velocity(nz, i, n, dx, lt, f, model, h[i], h[im], h[ip]);
}

}  // namespace

qew_status qew_rk_validate(qew_ctx *ctx, int n, const qew_params *p, const qew_rk_params *rp) {
    if (!p || !rp || n < 1) return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: bad arguments");
    if (n % 2 != 0)
        return qew_fail(ctx, QEW_ERR_ODD_LENGTH,
                        "rk_block: line length must be even for the red-black sweep");
    // The forward-zero march takes max_advance/dstep steps: it must be finite.
    if (!(rp->dstep > 0) || !std::isfinite(rp->max_advance) ||
        rp->max_advance / rp->dstep > 1e8 || rp->max_sweeps < 0)
        return qew_fail(ctx, QEW_ERR_INVALID,
                        "rk_block: need dstep > 0 and a finite max_advance/dstep <= 1e8");
    return QEW_OK;
}

// Host-driven rk_block: the reference's loop structure.
qew_status qew_rk_block_plain(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                              const qew_params *p, const qew_rk_params *rp, qew_rk_result *res,
                              int precision) {
    const double dx = p->physical_size / (double)n;
    QEW_TRY(qew_scratch_reserve(ctx, sizeof(double) * (size_t)n));
    double *adv = (double *)ctx->scratch;
    QEW_CUDA(ctx, cudaMemsetAsync(adv, 0, sizeof(double) * (size_t)n, ctx->stream));
    *res = qew_rk_result{};
    double mean_h0;
    QEW_TRY((vec_reduce<SumF, 1, false>(ctx, n, SumF{d_h}, &mean_h0)));
    mean_h0 /= (double)n;
    const RkP rk = rkp_from(rp);
    double cum_adv = 0;
    const int half = n / 2;
    for (int sweep = 0; sweep < rp->max_sweeps; ++sweep) {
        for (int color = 0; color < 2; ++color) {
            auto colour = [&](auto nz) -> qew_status {
                k_rk_colour<<<(half + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(
                    nz, d_h, adv, n, dx, p->line_tension, p->driving_force, p->model, color, rk);
                return qew_launch_check(ctx, "rk_colour");
            };
            QEW_TRY(precision == QEW_PREC_FP64_REFERENCE ? qew_dispatch_noise_ref(ctx, field, colour)
                                                          : qew_dispatch_noise(ctx, field, colour));
        }
        double total_adv;
        QEW_TRY((vec_reduce<SumF, 1, false>(ctx, n, SumF{adv}, &total_adv)));
        cum_adv += total_adv;
        const double mean_adv = cum_adv / (double)n;
        res->sweeps = sweep + 1;
        res->total_advance = total_adv;
        res->mean_h = mean_h0 + mean_adv;
        if (mean_adv > rp->runaway) {
            res->runaway = 1;
            res->blocked = 0;
            return QEW_OK;
        }
        if (total_adv < rp->sweep_tol) {
            res->blocked = 1;
            res->runaway = 0;
            return QEW_OK;
        }
    }
    res->blocked = 0;
    res->runaway = 0;
    return QEW_OK;
}

extern "C" {

qew_status qew_rk_site_velocity(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                                const qew_params *p, double *d_vel) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !p || !d_vel || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "rk_site_velocity: bad arguments");
    const double dx = p->physical_size / (double)n;
    return qew_dispatch_noise(ctx, field, [&](auto nz) -> qew_status {
        k_rk_velocity<<<(n + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(
            nz, d_h, n, dx, p->line_tension, p->driving_force, p->model, d_vel);
        return qew_launch_check(ctx, "rk_velocity");
    });
}

qew_status qew_rk_block(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                        const qew_params *p, const qew_rk_params *rp, qew_rk_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !res) return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: bad arguments");
    QEW_TRY(qew_rk_validate(ctx, n, p, rp));
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    return qew_rk_block_dispatch(ctx, field, d_h, n, p, rp, res);
}

qew_status qew_rk_block_form(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                             const qew_params *p, const qew_rk_params *rp, int form,
                             int precision, qew_rk_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !res) return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: bad arguments");
    QEW_TRY(qew_rk_validate(ctx, n, p, rp));
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (form == QEW_RK_PLAIN) {
        if (precision != QEW_PREC_FP64 && precision != QEW_PREC_FP64_REFERENCE)
            return qew_fail(ctx, QEW_ERR_UNSUPPORTED, "rk_block: the host-driven form is FP64 only");
        return qew_rk_block_plain(ctx, field, d_h, n, p, rp, res, precision);
    }
    if (form != QEW_RK_RESIDENT) return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: unknown form");
    return qew_rk_block_resident(ctx, field, d_h, n, p, rp, precision, res);
}

qew_status qew_depinning_bisect(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                const qew_params *p, const qew_rk_params *rp, double f_lo,
                                double f_hi, double rtol, int max_steps, double *f_c,
                                double *f_lo_out, double *f_hi_out, int *n_blocks) {
    return qew_depinning_bisect_prec(ctx, field, d_h, n, p, rp, f_lo, f_hi, rtol, max_steps,
                                     QEW_PREC_FP64, f_c, f_lo_out, f_hi_out, n_blocks);
}

qew_status qew_depinning_bisect_prec(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                     const qew_params *p, const qew_rk_params *rp, double f_lo,
                                     double f_hi, double rtol, int max_steps, int precision,
                                     double *f_c, double *f_lo_out, double *f_hi_out,
                                     int *n_blocks) {
    if (!f_c) return qew_fail(ctx, QEW_ERR_INVALID, "depinning_bisect: bad arguments");
    qew_bisect_result r;
    QEW_TRY(qew_depinning_bisect_ex(ctx, field, d_h, n, p, rp, f_lo, f_hi, rtol, max_steps,
                                    precision, &r, nullptr));
    *f_c = r.f_c;
    if (f_lo_out) *f_lo_out = r.f_lo;
    if (f_hi_out) *f_hi_out = r.f_hi;
    if (n_blocks) *n_blocks = r.blocks;
    return QEW_OK;
}

qew_status qew_depinning_bisect_ex(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                   const qew_params *p, const qew_rk_params *rp, double f_lo,
                                   double f_hi, double rtol, int max_steps, int precision,
                                   qew_bisect_result *res, int *h_verdicts) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !res || !(f_hi >= f_lo) || max_steps < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "depinning_bisect: bad arguments");
    QEW_TRY(qew_rk_validate(ctx, n, p, rp));
    *res = qew_bisect_result{};
    double *work = nullptr;
    QEW_TRY(qew_alloc_async(ctx, (void **)&work, sizeof(double) * (size_t)n));
    qew_params pp = *p;
    int steps = 0;
    qew_status st = QEW_OK;
    while ((f_hi - f_lo) > rtol * f_hi && steps < max_steps) {
        const double fm = 0.5 * (f_lo + f_hi);
        cudaError_t e = cudaMemcpyAsync(work, d_h, sizeof(double) * (size_t)n,
                                        cudaMemcpyDeviceToDevice, ctx->stream);
        if (e != cudaSuccess) {
            st = qew_fail(ctx, QEW_ERR_CUDA, "depinning_bisect: %s", cudaGetErrorString(e));
            break;
        }
        pp.driving_force = fm;
        qew_rk_result r;
        st = (precision == QEW_PREC_FP64) ? qew_rk_block_dispatch(ctx, field, work, n, &pp, rp, &r)
                                          : qew_rk_block_resident(ctx, field, work, n, &pp, rp,
                                                                  precision, &r);
        if (st != QEW_OK) break;
        const int verdict = r.blocked ? 0 : (r.runaway ? 1 : 2);
        if (h_verdicts) h_verdicts[steps] = verdict;
        ++steps;
        res->sweeps += r.sweeps;
        if (verdict == 0) {
            ++res->n_blocked;
            f_lo = fm;
            e = cudaMemcpyAsync(d_h, work, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice,
                                ctx->stream);
            if (e != cudaSuccess) {
                st = qew_fail(ctx, QEW_ERR_CUDA, "depinning_bisect: %s", cudaGetErrorString(e));
                break;
            }
        } else {
            if (verdict == 1)
                ++res->n_runaway;
            else
                ++res->n_timeout;
            res->f_hi_verdict = verdict;
            f_hi = fm;
        }
    }
    qew_free_async(work, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (st != QEW_OK) return st;
    res->f_c = 0.5 * (f_lo + f_hi);
    res->f_lo = f_lo;
    res->f_hi = f_hi;
    res->blocks = steps;
    return QEW_OK;
}

}  // extern "C"
