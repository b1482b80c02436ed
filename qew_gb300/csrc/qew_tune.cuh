// qew_tune.cuh -- the launch-shape autotuner.
//
// A kernel with several launch shapes that give bitwise-identical results
// (sites per thread, resident CTAs per SM, the Rosso-Krauth search width)
// asks qew_tune_pick for its shape. On the first call of a (device, kernel,
// shape class) the tuner times every candidate on that call's own work with
// CUDA events on the context's stream (one warm-up launch, then the best of
// a few timed launches each) and caches the fastest for the process; later
// calls of the class take the cached choice without timing. A context may
// switch tuning off (the hand-chosen default shape is used) or force one
// candidate (tests run every candidate this way).
#pragma once

#include <string>
#include <vector>

#include "qew_internal.cuh"

enum {
    kTuneGradientPoly = 0,   // k_gradient_poly: sites per thread x resident CTAs per SM
    kTuneGradientSplit = 1,  // k_gradient_split_persist: sites per thread x resident CTAs per SM
    kTuneRkSearch = 2,       // k_rk_resident: lanes per site's forward-zero search
    kTuneLangevinRun = 3,    // k_langevin_run / k_langevin_run_tb: steps per grid barrier x CTAs per SM
    kTuneKernels = 4
};

// Shape class of a launch over `points` work items (log2 bucket) with a
// kernel-specific variant in [0, 8).
int qew_tune_class(long long points, int variant);

// Cached choice, or -1.
int qew_tune_cached(int device, int kernel, int cls);
void qew_tune_remember(int device, int kernel, int cls, int choice, const std::string &detail);

// Chooses the candidate for this call. run(c) enqueues candidate c's launch
// on ctx->stream and returns its status; `names[c]` describes candidate c.
// When the choice is made by timing, every candidate runs on the call's
// work, so each candidate must leave outputs that a later run overwrites
// completely (or work on a copy).
// A candidate replaces the default only when it is faster by more than
// `margin` (a fraction of the default's time): 0 for timing runs that repeat
// the call's own work exactly, more where the timed work only samples it.
template <class Run>
qew_status qew_tune_pick(qew_ctx *ctx, int kernel, int cls, int ncand, int default_cand,
                         const char *const *names, Run &&run, int *chosen,
                         float margin = 0.0f) {
    if (ctx->tune_force[kernel] >= 0 && ctx->tune_force[kernel] < ncand) {
        *chosen = ctx->tune_force[kernel];
        return QEW_OK;
    }
    if (!ctx->autotune || ncand <= 1) {
        *chosen = default_cand;
        return QEW_OK;
    }
    const int c0 = qew_tune_cached(ctx->device, kernel, cls);
    if (c0 >= 0 && c0 < ncand) {
        *chosen = c0;
        return QEW_OK;
    }
    cudaEvent_t e0, e1;
    QEW_CUDA(ctx, cudaEventCreate(&e0));
    QEW_CUDA(ctx, cudaEventCreate(&e1));
    int best = default_cand;
    float best_ms = 3.4e38f;
    std::vector<float> times(ncand, 3.4e38f);
    std::string detail;
    qew_status st = QEW_OK;
    for (int c = 0; c < ncand && st == QEW_OK; ++c) {
        st = run(c);  // warm-up
        float cand_ms = 3.4e38f;
        for (int rep = 0; rep < 3 && st == QEW_OK; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            st = run(c);
            cudaEventRecord(e1, ctx->stream);
            if (st != QEW_OK) break;
            float ms = 0.f;
            if (cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                st = qew_fail(ctx, QEW_ERR_CUDA, "autotune: event timing failed");
                break;
            }
            if (ms < cand_ms) cand_ms = ms;
        }
        if (st == QEW_OK) {
            char buf[160];
            snprintf(buf, sizeof(buf), "%s%s %.1f us", c ? "; " : "", names[c], 1e3 * cand_ms);
            detail += buf;
            times[c] = cand_ms;
            if (cand_ms < best_ms) {
                best_ms = cand_ms;
                best = c;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != QEW_OK) return st;
    if (best != default_cand && !(best_ms < (1.0f - margin) * times[default_cand]))
        best = default_cand;
    qew_tune_remember(ctx->device, kernel, cls, best, detail);
    *chosen = best;
    return QEW_OK;
}
