// qew_ensemble.cu -- batched statics: thousands of independent lines of
// uneven length relaxed by one persistent kernel (no reference counterpart;
// the reference relaxes one line per lbfgs_minimize call, lbfgs.h:94-287,
// and realisations are separate process runs).
//
// Each CTA of a persistent grid takes the next line from a queue ordered by
// decreasing length (longest first, so the tail of the launch is short
// lines) and runs, inside the CTA, the complete lbfgs_minimize twice:
//   1. on the FP32 split-index gather (FP32 coefficients), with the FP64
//      vectors, dot products and Armijo search of the reference, until
//      max|g| < ftol_fp32;
//   2. from that point with a fresh history on the FP64 gather, until the
//      caller's FP64 tolerance (the refinement).
// A CTA's workspace is reused by every line it processes, so the device
// memory held is (CTAs x longest line), independent of the line count.
#include <algorithm>
#include <numeric>
#include <vector>

#include "qew_lbfgs_internal.cuh"
#include "qew_lbfgs_resident.cuh"
#include "qew_noise32.cuh"

namespace {

constexpr int kEnsBS = 512;

struct EnsJob {
    const double *coef64;
    const double *poly64;  // FP64 cell-polynomial store, or null
    int ky;                // y * 2^ky == y / dy, or kPolyNotPow2
#ifdef QEW_BOUNDS_CHECK
    unsigned long long *oob;
#endif
    const float *coef32;
    const float *edge32;
    int nx, ny;
    double fdx, fdy, Lx;
    double *h;
    int n;
    qew_params p;
    PrecondCoef pc;
};

__device__ __forceinline__ NoiseBSpline64 job_noise64(const EnsJob &j) {
    NoiseBSpline64 nz;
    nz.coef = j.coef64;
    nz.nx = j.nx;
    nz.ny = j.ny;
    nz.dx = j.fdx;
    nz.dy = j.fdy;
    nz.inv_dx = 1.0 / j.fdx;
    nz.inv_dy = 1.0 / j.fdy;
    nz.dx_pow2 = dbl_is_pow2(j.fdx);
    nz.dy_pow2 = dbl_is_pow2(j.fdy);
    nz.xconst = (j.n == j.nx && j.p.physical_size == j.Lx && nz.dx_pow2);
    nz.wxc[0] = 0.125 * (1.0 / 6.0);  // bsw_value(1/2), as NoiseBSpline64::wxc
    nz.wxc[1] = 2.875 * (1.0 / 6.0);
    nz.wxc[2] = 2.875 * (1.0 / 6.0);
    nz.wxc[3] = 0.125 * (1.0 / 6.0);
    nz.poly = (j.n == j.nx && j.p.physical_size == j.Lx) ? j.poly64 : nullptr;
    nz.ky = j.ky;
#ifdef QEW_BOUNDS_CHECK
    nz.oob = j.oob;
#endif
    return nz;
}

__device__ __forceinline__ NoiseSplit32 job_noise32(const EnsJob &j) {
    NoiseSplit32 nz;
    nz.coef = j.coef32;
    nz.nx = j.nx;
    nz.ny = j.ny;
    nz.dx = j.fdx;
    nz.dy = j.fdy;
    nz.inv_dx = 1.0 / j.fdx;
    nz.inv_dy = 1.0 / j.fdy;
    nz.dx_pow2 = dbl_is_pow2(j.fdx);
    nz.dy_pow2 = dbl_is_pow2(j.fdy);
    nz.xconst = (j.n == j.nx && j.p.physical_size == j.Lx && nz.dx_pow2);
    nz.edge = nz.xconst ? j.edge32 : nullptr;
    nz.inv_dy_f = (float)(1.0 / j.fdy);
#ifdef QEW_BOUNDS_CHECK
    nz.oob = j.oob;
#endif
    return nz;
}

__global__ void __launch_bounds__(kEnsBS, 2)
k_ensemble(const EnsJob *__restrict__ jobs, const int *__restrict__ order, int count,
           unsigned int *next, LbfgsCfg cfg32, LbfgsCfg cfg64, int use32, double *ws_base,
           size_t ws_per_cta, size_t npad_max, qew_lbfgs_result *results) {
    __shared__ int s_job;
    double *ws = ws_base + (size_t)blockIdx.x * ws_per_cta;
    for (;;) {  // bounded: every pass takes a new queue ticket
        if (threadIdx.x == 0) s_job = (int)atomicAdd(next, 1u);
        __syncthreads();
        const int k = s_job;
        __syncthreads();
        if (k >= count) break;
        const int id = order[k];
        const EnsJob j = jobs[id];
        const size_t npad = ((size_t)j.n + 31) & ~size_t(31);
        (void)npad_max;
        qew_lbfgs_result r32{};
        if (use32) r32 = lbfgs_block<NoiseSplit32, kEnsBS, float>(job_noise32(j), j.h, j.n, j.p, cfg32, j.pc, ws, npad);
        qew_lbfgs_result r = lbfgs_block<NoiseBSpline64, kEnsBS>(job_noise64(j), j.h, j.n, j.p, cfg64, j.pc, ws, npad);
        if (threadIdx.x == 0) {
            r.iterations += r32.iterations;
            r.n_func_evals += r32.n_func_evals;
            r.n_curvature_skips += r32.n_curvature_skips;
            r.n_ls_restarts += r32.n_ls_restarts;
            results[id] = r;
        }
        __syncthreads();
    }
}

}  // namespace

extern "C" qew_status qew_ensemble_minimize(qew_ctx *ctx, int count, const qew_ensemble_line *lines,
                                            const qew_ensemble_params *ep,
                                            qew_lbfgs_result *results) {
    QEW_RANGE();
    if (!ctx || count < 0 || (count > 0 && (!lines || !results)) || !ep)
        return qew_fail(ctx, QEW_ERR_INVALID, "ensemble_minimize: bad arguments");
    if (count == 0) return QEW_OK;
    const qew_lbfgs_params &lp = ep->lbfgs;
    if (lp.m < 1 || lp.m > kLbfgsMaxM || lp.max_ls < 0 || lp.max_iter < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "ensemble_minimize: need 1 <= m <= %d", kLbfgsMaxM);
    const int use32 = ep->ftol_fp32 > 0 ? 1 : 0;
    std::vector<EnsJob> jobs(count);
    int nmax = 0;
    for (int k = 0; k < count; ++k) {
        const qew_ensemble_line &L = lines[k];
        const qew_field *f = L.field;
        if (!f || !L.d_h || L.n < 1 || f->kind != QEW_FIELD_BSPLINE || !f->coef64 ||
            (use32 && !f->coef32))
            return qew_fail(ctx, QEW_ERR_INVALID,
                            "ensemble_minimize: line %d needs a B-spline field with FP64%s "
                            "coefficients", k, use32 ? " and FP32" : "");
        EnsJob &j = jobs[k];
        j.coef64 = f->coef64;
        j.poly64 = f->poly64;
        j.ky = make_bspline64(f).ky;
#ifdef QEW_BOUNDS_CHECK
        j.oob = qew_bounds_words();
#endif
        j.coef32 = f->coef32;
        j.edge32 = f->edge32;
        j.nx = f->nx;
        j.ny = f->ny;
        j.fdx = f->dx;
        j.fdy = f->dy;
        j.Lx = f->Lx;
        j.h = L.d_h;
        j.n = L.n;
        j.p = L.p;
        j.pc = lp.precondition ? qew_precond_coef(L.n, L.p.line_tension, L.p.physical_size,
                                                  L.precond_shift)
                               : PrecondCoef{};
        nmax = std::max(nmax, L.n);
    }
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return jobs[a].n > jobs[b].n; });

    int per_sm = 0;
    QEW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ensemble, kEnsBS, 0));
    const int grid = std::max(1, std::min(count, ctx->num_sms * std::max(per_sm, 1)));
    const size_t npad_max = ((size_t)nmax + 31) & ~size_t(31);
    const size_t ws_per_cta = npad_max * (size_t)(kLbfgsVecs + 2 * (lp.m + 1));
    // layout: [ws (grid x ws_per_cta doubles)][jobs][order][results][counter]
    const size_t off_jobs = ((ws_per_cta * grid * sizeof(double)) + 255) & ~size_t(255);
    const size_t off_order = (off_jobs + sizeof(EnsJob) * count + 255) & ~size_t(255);
    const size_t off_res = (off_order + sizeof(int) * count + 255) & ~size_t(255);
    const size_t off_cnt = (off_res + sizeof(qew_lbfgs_result) * count + 255) & ~size_t(255);
    QEW_TRY(qew_scratch_reserve(ctx, off_cnt + 256));
    char *base = (char *)ctx->scratch;
    EnsJob *d_jobs = (EnsJob *)(base + off_jobs);
    int *d_order = (int *)(base + off_order);
    qew_lbfgs_result *d_res = (qew_lbfgs_result *)(base + off_res);
    unsigned int *d_cnt = (unsigned int *)(base + off_cnt);
    QEW_CUDA(ctx, cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(EnsJob) * count,
                                  cudaMemcpyHostToDevice, ctx->stream));
    QEW_CUDA(ctx, cudaMemcpyAsync(d_order, order.data(), sizeof(int) * count,
                                  cudaMemcpyHostToDevice, ctx->stream));
    QEW_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, sizeof(unsigned int), ctx->stream));
    LbfgsCfg cfg64 = lbfgs_cfg_from(&lp);
    LbfgsCfg cfg32 = cfg64;
    cfg32.ftol = ep->ftol_fp32;
    cfg32.max_iter = ep->max_iter_fp32 > 0 ? ep->max_iter_fp32 : lp.max_iter;
    k_ensemble<<<grid, kEnsBS, 0, ctx->stream>>>(d_jobs, d_order, count, d_cnt, cfg32, cfg64, use32,
                                                  (double *)base, ws_per_cta, npad_max, d_res);
    QEW_TRY(qew_launch_check(ctx, "ensemble"));
    QEW_CUDA(ctx, cudaMemcpyAsync(results, d_res, sizeof(qew_lbfgs_result) * count,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

// ------------------------------------------------------------ serving lane
// A device-resident request loop for static lines (qew_serve_lane.cuh): a
// persistent grid whose CTAs claim jobs from a ring in mapped host memory as
// the host publishes them, relax each like one ensemble line (FP32 phase,
// FP64 refinement), and post the result back to the ring. Every wait is
// bounded: a CTA that finds no work for idle_polls polls leaves, and the
// host relaunches the grid when jobs remain unclaimed.
#include "qew_serve_lane.cuh"

namespace {

struct LaneRing {  // mapped pinned host memory
    EnsJob jobs[kLaneRing];
    qew_lbfgs_result results[kLaneRing];
    unsigned long long done[kLaneRing];  // k + 1 once job k's result is posted
    unsigned int published;              // jobs [0, published) are readable
    int closing;                         // set by the host to let the grid leave
};
static_assert(sizeof(EnsJob) % 8 == 0, "EnsJob is copied in 8-byte words");

__device__ __forceinline__ unsigned int ld_acquire_sys_u32(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__global__ void __launch_bounds__(kEnsBS, 2)
k_serve_static(LaneRing *ring, unsigned int *head, LbfgsCfg cfg32, LbfgsCfg cfg64, int use32,
               double *ws_base, size_t ws_per_cta, long long idle_polls) {
    __shared__ int s_k;
    __shared__ EnsJob s_job;
    double *ws = ws_base + (size_t)blockIdx.x * ws_per_cta;
    for (;;) {  // each pass claims one job or leaves; a solve is bounded by max_iter
        if (threadIdx.x == 0) {
            int k = -1;
            long long polls = 0;
            while (polls <= idle_polls) {
                const unsigned int pub = ld_acquire_sys_u32(&ring->published);
                const unsigned int h = *(volatile unsigned int *)head;
                if (h < pub) {
                    if (atomicCAS(head, h, h + 1u) == h) {
                        k = (int)h;
                        break;
                    }
                    ++polls;  // another CTA took it: counts toward the bound
                    continue;
                }
                if (*(volatile int *)&ring->closing) break;
                ++polls;
                __nanosleep(1000);
            }
            if (k >= 0) {
                const volatile unsigned long long *src =
                    (const volatile unsigned long long *)&ring->jobs[k % kLaneRing];
                unsigned long long *dst = (unsigned long long *)&s_job;
                for (int w = 0; w < (int)(sizeof(EnsJob) / 8); ++w) dst[w] = src[w];
            }
            s_k = k;
        }
        __syncthreads();
        const int k = s_k;
        if (k < 0) break;
        const EnsJob j = s_job;
        __syncthreads();
        const size_t npad = ((size_t)j.n + 31) & ~size_t(31);
        qew_lbfgs_result r32{};
        if (use32)
            r32 = lbfgs_block<NoiseSplit32, kEnsBS, float>(job_noise32(j), j.h, j.n, j.p, cfg32,
                                                           j.pc, ws, npad);
        qew_lbfgs_result r =
            lbfgs_block<NoiseBSpline64, kEnsBS>(job_noise64(j), j.h, j.n, j.p, cfg64, j.pc, ws, npad);
        if (threadIdx.x == 0) {
            r.iterations += r32.iterations;
            r.n_func_evals += r32.n_func_evals;
            r.n_curvature_skips += r32.n_curvature_skips;
            r.n_ls_restarts += r32.n_ls_restarts;
            ring->results[k % kLaneRing] = r;
            __threadfence_system();
            *(volatile unsigned long long *)&ring->done[k % kLaneRing] =
                (unsigned long long)k + 1ull;
        }
        __syncthreads();
    }
}

}  // namespace

struct StaticLane {
    int device = 0;
    cudaStream_t stream = nullptr;  // the lane kernel's stream
    LaneRing *ring = nullptr;       // host address
    LaneRing *ring_d = nullptr;     // device address of the same memory
    unsigned int *head = nullptr;   // device: jobs claimed so far
    double *ws = nullptr;
    size_t ws_per_cta = 0;
    int grid = 0, nmax = 0, use32 = 0;
    LbfgsCfg cfg32{}, cfg64{};
    long long idle_polls = 1 << 14;  // about 16 ms of polls without work
    cudaEvent_t done_ev = nullptr;
    bool running = false;
    unsigned int published = 0;
    uint64_t launches = 0;
};

qew_status qew_lane_create(int device, int nmax, const qew_lbfgs_params *lp, double ftol32,
                           int ctas, StaticLane **out) {
    if (!out || !lp || nmax < 1 || ctas < 1 || lp->m < 1 || lp->m > kLbfgsMaxM)
        return QEW_ERR_INVALID;
    StaticLane *L = new (std::nothrow) StaticLane();
    if (!L) return QEW_ERR_NOMEM;
    L->device = device;
    L->nmax = nmax;
    L->grid = ctas;
    L->use32 = ftol32 > 0 ? 1 : 0;
    L->cfg64 = lbfgs_cfg_from(lp);
    L->cfg32 = L->cfg64;
    L->cfg32.ftol = ftol32;
    const size_t npad_max = ((size_t)nmax + 31) & ~size_t(31);
    L->ws_per_cta = npad_max * (size_t)(kLbfgsVecs + 2 * (lp->m + 1));
    auto fail = [&](qew_status s) {
        if (L->ws) cudaFree(L->ws);
        if (L->head) cudaFree(L->head);
        if (L->ring) cudaFreeHost(L->ring);
        if (L->stream) cudaStreamDestroy(L->stream);
        if (L->done_ev) cudaEventDestroy(L->done_ev);
        cudaGetLastError();
        delete L;
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&L->done_ev, cudaEventDisableTiming) != cudaSuccess)
        return fail(QEW_ERR_CUDA);
    if (cudaHostAlloc((void **)&L->ring, sizeof(LaneRing), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void **)&L->ring_d, L->ring, 0) != cudaSuccess ||
        cudaMalloc((void **)&L->head, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc((void **)&L->ws, L->ws_per_cta * (size_t)ctas * sizeof(double)) != cudaSuccess)
        return fail(QEW_ERR_NOMEM);
    memset((void *)L->ring, 0, sizeof(LaneRing));
    if (cudaMemset(L->head, 0, sizeof(unsigned int)) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return fail(QEW_ERR_CUDA);
    *out = L;
    return QEW_OK;
}

qew_status qew_lane_publish(StaticLane *L, const qew_field *f, double *d_h, int n,
                            const qew_params *p, double shift, unsigned int *k) {
    if (!L || !f || !d_h || !p || n < 1 || n > L->nmax || f->kind != QEW_FIELD_BSPLINE ||
        !f->coef64 || (L->use32 && !f->coef32))
        return QEW_ERR_INVALID;
    EnsJob j{};
    j.coef64 = f->coef64;
    j.poly64 = f->poly64;
    j.ky = make_bspline64(f).ky;
#ifdef QEW_BOUNDS_CHECK
    j.oob = qew_bounds_words();
#endif
    j.coef32 = f->coef32;
    j.edge32 = f->edge32;
    j.nx = f->nx;
    j.ny = f->ny;
    j.fdx = f->dx;
    j.fdy = f->dy;
    j.Lx = f->Lx;
    j.h = d_h;
    j.n = n;
    j.p = *p;
    j.pc = L->cfg64.precondition ? qew_precond_coef(n, p->line_tension, p->physical_size, shift)
                                 : PrecondCoef{};
    const unsigned int idx = L->published;
    L->ring->jobs[idx % kLaneRing] = j;
    __atomic_store_n(&L->ring->published, idx + 1u, __ATOMIC_RELEASE);
    L->published = idx + 1u;
    *k = idx;
    return QEW_OK;
}

qew_status qew_lane_pump(StaticLane *L, cudaStream_t aux) {
    if (!L) return QEW_ERR_INVALID;
    if (L->running) {
        const cudaError_t q = cudaEventQuery(L->done_ev);
        if (q == cudaErrorNotReady) return QEW_OK;
        if (q != cudaSuccess) return QEW_ERR_CUDA;
        L->running = false;
    }
    unsigned int claimed = 0;
    if (cudaMemcpyAsync(&claimed, L->head, sizeof(unsigned int), cudaMemcpyDeviceToHost, aux) !=
            cudaSuccess ||
        cudaStreamSynchronize(aux) != cudaSuccess)
        return QEW_ERR_CUDA;
    if (claimed >= L->published) return QEW_OK;  // nothing waits
    k_serve_static<<<L->grid, kEnsBS, 0, L->stream>>>(L->ring_d, L->head, L->cfg32, L->cfg64,
                                                      L->use32, L->ws, L->ws_per_cta,
                                                      L->idle_polls);
    if (cudaGetLastError() != cudaSuccess) return QEW_ERR_CUDA;
    if (cudaEventRecord(L->done_ev, L->stream) != cudaSuccess) return QEW_ERR_CUDA;
    L->running = true;
    ++L->launches;
    return QEW_OK;
}

bool qew_lane_done(StaticLane *L, unsigned int k, qew_lbfgs_result *r) {
    const unsigned long long d = __atomic_load_n(&L->ring->done[k % kLaneRing], __ATOMIC_ACQUIRE);
    if (d != (unsigned long long)k + 1ull) return false;
    *r = L->ring->results[k % kLaneRing];
    return true;
}

uint64_t qew_lane_launches(const StaticLane *L) { return L ? L->launches : 0; }

void qew_lane_destroy(StaticLane *L) {
    if (!L) return;
    cudaSetDevice(L->device);
    __atomic_store_n(&L->ring->closing, 1, __ATOMIC_RELEASE);
    cudaStreamSynchronize(L->stream);  // every CTA leaves at its next idle check
    cudaFree(L->ws);
    cudaFree(L->head);
    cudaFreeHost(L->ring);
    cudaEventDestroy(L->done_ev);
    cudaStreamDestroy(L->stream);
    delete L;
}
