// qew_rk_resident.cu -- rk_block (rosso_krauth.h:128-194) as one persistent
// cooperative kernel: all sweeps, both colours and the per-sweep verdict run
// on the device, with a grid barrier between colours instead of a kernel
// launch, and the sweep's total advance reduced deterministically (per-CTA
// partials summed in CTA order by every CTA). Each site's forward zero is
// evaluated by a group of lanes (rk_forward_zero_group: several march points
// or bisection levels per round) that replays the serial search exactly, so
// both forms produce bit-identical lines.
//
// The grid barrier spins on a generation word with a bounded number of polls;
// if it gives up it raises an error flag, every CTA leaves the sweep loop, and
// the host returns QEW_ERR_TIMEOUT. A cooperative launch guarantees that all
// CTAs are resident, so the barrier completes unless the device is stalled.
#include <cooperative_groups.h>

#include <algorithm>

#include "qew_gridsync.cuh"
#include "qew_tune.cuh"
#include "qew_internal.cuh"
#include "qew_noise32.cuh"
#include "qew_rk_device.cuh"
#include "qew_rk_internal.cuh"

namespace {

constexpr int kRkBS = 32;  // one warp per CTA: a 16384-site line still spreads over every SM
#ifndef QEW_RK_WARPS_PER_SM
#define QEW_RK_WARPS_PER_SM 4  // build-time tuning knob (measured on GB300)
#endif
// kRkGroup lanes per site (8: 7 march points or 3 bisection levels per round;
// 4: 3 points or 2 levels; 2: the serial search with each velocity's two
// gathers on the two lanes; 1: the serial search). All widths give the same
// result; the launch picks one by the budgets below.
template <class Noise, int kRkGroup>
__global__ void __launch_bounds__(kRkBS)
k_rk_resident(Noise nz, double *__restrict__ h, double *__restrict__ adv, int n, double dx,
              double lt, double f, int model, RkP rp, double *partials, GridSync *sync,
              qew_rk_result *out) {
    const unsigned int nb = gridDim.x;
    const int gtid = blockIdx.x * kRkBS + threadIdx.x;
    const int gstride = nb * kRkBS;
    const int half = n / 2;
    const int glane = threadIdx.x & (kRkGroup - 1);
    const unsigned gmask = ((kRkGroup == 32) ? 0xffffffffu : ((1u << kRkGroup) - 1u))
                           << ((threadIdx.x & 31) & ~(kRkGroup - 1));
    __shared__ double s_w[kRkBS / 32];
    // mean(h) at entry (rosso_krauth.h:144-148)
    double acc = 0.0;
    for (int i = gtid; i < n; i += gstride) acc += h[i];
    acc = block_sum<kRkBS>(acc, s_w);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
    if (!grid_sync_bounded(sync, nb)) return;
    double mean_h0 = 0.0;
    for (unsigned int b = 0; b < nb; ++b) mean_h0 += __ldcg(partials + b);
    mean_h0 /= (double)n;

    qew_rk_result res{};
    double cum_adv = 0.0;
    for (int sweep = 0; sweep < rp.max_sweeps; ++sweep) {
        double local = 0.0;
        for (int color = 0; color < 2; ++color) {
            // one group of kRkGroup lanes per site of this colour
            for (int k = gtid / kRkGroup; k < half; k += gstride / kRkGroup) {
                const int i = 2 * k + color;
                const int im = (i == 0) ? n - 1 : i - 1;
                const int ip = (i + 1 == n) ? 0 : i + 1;
                bool found = false;
                const double hi = __ldcg(h + i);
                double hnew;
                if constexpr (kRkGroup == 1) {
                    hnew = rk_forward_zero(nz, i, n, dx, lt, f, model, hi, __ldcg(h + im),
                                           __ldcg(h + ip), rp, found);
                } else if constexpr (kRkGroup == 2) {
                    hnew = rk_forward_zero_pair(nz, i, n, dx, lt, f, model, hi, __ldcg(h + im),
                                                __ldcg(h + ip), rp, found, glane, gmask);
                    __syncwarp(gmask);  // both lanes have read h[i]
                } else {
                    hnew = rk_forward_zero_group<kRkGroup>(nz, i, n, dx, lt, f, model, hi,
                                                          __ldcg(h + im), __ldcg(h + ip), rp,
                                                          found, glane, gmask);
                    __syncwarp(gmask);  // every lane has read h[i]
                }
                if (glane == 0) {
                    const double a = hnew - hi;
                    adv[i] = a;
                    h[i] = hnew;
                    local += a;
                }
            }
            if (color == 0 && !grid_sync_bounded(sync, nb)) return;
        }
        // sweep total: per-CTA partials (double-buffered by sweep parity)
        double *part = partials + nb * (1 + (sweep & 1));
        local = block_sum<kRkBS>(local, s_w);
        if (threadIdx.x == 0) part[blockIdx.x] = local;
        if (!grid_sync_bounded(sync, nb)) return;
        double total_adv = 0.0;
        for (unsigned int b = 0; b < nb; ++b) total_adv += __ldcg(part + b);
        cum_adv += total_adv;
        const double mean_adv = cum_adv / (double)n;
        res.sweeps = sweep + 1;
        res.total_advance = total_adv;
        res.mean_h = mean_h0 + mean_adv;
        if (mean_adv > rp.runaway) {
            res.runaway = 1;
            res.blocked = 0;
            break;
        }
        if (total_adv < rp.sweep_tol) {
            res.blocked = 1;
            res.runaway = 0;
            break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = res;
}

}  // namespace

qew_status qew_rk_block_resident(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                 const qew_params *p, const qew_rk_params *rp, int precision,
                                 qew_rk_result *res) {
    const double dx = p->physical_size / (double)n;
    const RkP rk = rkp_from(rp);
    auto launch = [&](auto nz) -> qew_status {
        using N = decltype(nz);
        // The search width: wider groups shorten each site's chain of
        // dependent evaluations but multiply its FP64 work, which pays only
        // while the SMs' FP64 pipes idle; lane pairs split each evaluation's
        // two gathers (the same FP64 work in half the chain). Each form has a
        // warps-per-SM budget (and the resident slots, or the context's share
        // of them); the serial form takes what is left.
        // Measured (sweeps/s, bitwise-equal results): 8-lane groups win while
        // they stay within about 2 warps per SM, lane pairs up to about 4,
        // the serial search beyond; 4-lane groups were never the best.
        const void *forms[3] = {(const void *)k_rk_resident<N, 8>, (const void *)k_rk_resident<N, 2>,
                                (const void *)k_rk_resident<N, 1>};
        const int sizes[3] = {8, 2, 1};
        const long long warps_per_sm[3] = {QEW_RK_WARPS_PER_SM / 2, QEW_RK_WARPS_PER_SM, 0};
        const long long half = n / 2;
        int grids[3];
        int heuristic = 2, grid_max = 1;
        for (int k = 0; k < 3; ++k) {
            int per_sm = 0;
            QEW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, forms[k], kRkBS, 0));
            int slots = ctx->num_sms * std::max(per_sm, 1);
            if (ctx->warp_cap > 0) slots = std::min(slots, ctx->warp_cap / (kRkBS / 32));
            const long long budget = std::min<long long>(slots, warps_per_sm[k] * ctx->num_sms);
            const long long want = (half * sizes[k] + kRkBS - 1) / kRkBS;
            grids[k] = (int)std::max(1LL, std::min(want, (long long)std::max(slots, 1)));
            grid_max = std::max(grid_max, grids[k]);
            if (heuristic == 2 && k < 2 && want <= budget) heuristic = k;
        }
        // scratch: adv[n], partials[3*grid], sync word, result
        const size_t off_part = ((size_t)n * sizeof(double) + 255) & ~size_t(255);
        const size_t off_sync = (off_part + 3 * (size_t)grid_max * sizeof(double) + 255) & ~size_t(255);
        const size_t off_res = (off_sync + sizeof(GridSync) + 255) & ~size_t(255);
        QEW_TRY(qew_scratch_reserve(ctx, off_res + sizeof(qew_rk_result) + 256));
        char *base = (char *)ctx->scratch;
        double *adv = (double *)base;
        double *part = (double *)(base + off_part);
        GridSync *sync = (GridSync *)(base + off_sync);
        qew_rk_result *d_res = (qew_rk_result *)(base + off_res);
        double lt = p->line_tension, fd = p->driving_force;
        int model = p->model;
        auto run_form = [&](int k, double *hp, RkP rkk) -> qew_status {
            QEW_CUDA(ctx, cudaMemsetAsync(adv, 0, (size_t)n * sizeof(double), ctx->stream));
            QEW_TRY(qew_gridsync_init(ctx, sync));
            void *args[] = {(void *)&nz, (void *)&hp, (void *)&adv, (void *)&n, (void *)&dx,
                            (void *)&lt, (void *)&fd, (void *)&model, (void *)&rkk,
                            (void *)&part, (void *)&sync, (void *)&d_res};
            QEW_CUDA(ctx, cudaLaunchCooperativeKernel(forms[k], dim3(grids[k]), dim3(kRkBS), args,
                                                      0, ctx->stream));
            return qew_launch_check(ctx, "rk_resident");
        };
        // The search width: the autotuner times the three widths on the first
        // call of a (line length, noise form, GPU share) class, each on a copy
        // of this call's line for a few sweeps (every width gives the same
        // lines bit for bit); the budget rule above is the default, replaced
        // only by a width more than 20 % faster (a few sweeps sample a block
        // whose work per sweep changes as it creeps).
        static const char *const names[3] = {"8-lane groups", "lane pairs", "one lane"};
        int noise_kind = 0;
        if constexpr (std::is_same<N, NoiseSplit32>::value) noise_kind = 3;
        else if constexpr (noise_is_ref<N>::value) noise_kind = 2;
        else if constexpr (std::is_same<N, NoiseBSpline64>::value) noise_kind = nz.poly ? 1 : 0;
        // The first sweeps of a block move many sites a long way (FP64-heavy)
        // and the later ones few (latency-bound), and a block spends most of
        // its sweeps in the later phase: the probe line is first advanced 24
        // sweeps with the default width, then every candidate is timed for 8
        // sweeps from that state.
        double *tune_h = nullptr, *tune_start = nullptr;
        RkP rk_probe = rk, rk_advance = rk;
        rk_probe.max_sweeps = std::min(rk.max_sweeps, 8);
        rk_advance.max_sweeps = std::min(rk.max_sweeps, 24);
        auto probe = [&](int k) -> qew_status {
            if (!tune_h) {
                QEW_TRY(qew_alloc_async(ctx, (void **)&tune_h, (size_t)n * sizeof(double)));
                QEW_TRY(qew_alloc_async(ctx, (void **)&tune_start, (size_t)n * sizeof(double)));
                QEW_CUDA(ctx, cudaMemcpyAsync(tune_start, d_h, (size_t)n * sizeof(double),
                                              cudaMemcpyDeviceToDevice, ctx->stream));
                QEW_TRY(run_form(heuristic, tune_start, rk_advance));
            }
            QEW_CUDA(ctx, cudaMemcpyAsync(tune_h, tune_start, (size_t)n * sizeof(double),
                                          cudaMemcpyDeviceToDevice, ctx->stream));
            return run_form(k, tune_h, rk_probe);
        };
        int cand = heuristic;
        const qew_status ts =
            qew_tune_pick(ctx, kTuneRkSearch,
                          qew_tune_class(n, 2 * noise_kind + (ctx->warp_cap > 0 ? 1 : 0)), 3,
                          heuristic, names, probe, &cand, 0.2f);
        if (tune_h) qew_free_async(tune_h, ctx->stream);
        if (tune_start) qew_free_async(tune_start, ctx->stream);
        QEW_TRY(ts);
        QEW_TRY(run_form(cand, d_h, rk));
        GridSync hs;
        QEW_CUDA(ctx, cudaMemcpyAsync(res, d_res, sizeof(qew_rk_result), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        QEW_CUDA(ctx, cudaMemcpyAsync(&hs, sync, sizeof(GridSync), cudaMemcpyDeviceToHost, ctx->stream));
        QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (hs.err) return qew_fail(ctx, QEW_ERR_TIMEOUT, "rk_block: grid barrier timed out");
        return QEW_OK;
    };
    if (precision == QEW_PREC_FP32_SPLIT) {
        if (field->kind != QEW_FIELD_BSPLINE || !field->coef32)
            return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: FP32 storage needs QEW_STORE_FP32");
        return launch(make_split32(field, n, p->physical_size));
    }
    if (precision == QEW_PREC_FP64_REFERENCE) return qew_dispatch_noise_ref(ctx, field, launch);
    if (precision != QEW_PREC_FP64)
        return qew_fail(ctx, QEW_ERR_INVALID, "rk_block: unknown precision %d", precision);
    return qew_dispatch_noise(ctx, field, launch, n, p->physical_size);
}

qew_status qew_rk_block_dispatch(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                                 const qew_params *p, const qew_rk_params *rp,
                                 qew_rk_result *res) {
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
    if (!coop) return qew_rk_block_plain(ctx, field, d_h, n, p, rp, res, QEW_PREC_FP64);
    return qew_rk_block_resident(ctx, field, d_h, n, p, rp, QEW_PREC_FP64, res);
}
