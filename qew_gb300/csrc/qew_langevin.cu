// qew_langevin.cu -- overdamped Langevin / Euler-Maruyama step
// (LangevinDynamics, dynamics.h:27-70): h_i += -drift * dE/dh_i + diff * xi_i.
//
// The reference draws xi from Kokkos' Random_XorShift64_Pool, whose stream is
// specific to that library; here xi comes from a Philox4x32-10 counter stream
// keyed by (seed, site pair, step), so any step of any site can be regenerated
// independently (and by the oracle, bit-for-bit in the uniforms). Trajectory
// parity with the reference is checked through the increments entry point,
// which takes xi from the caller.
#include <algorithm>
#include <climits>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>

#include "qew_gridsync.cuh"
#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"
#include "qew_noise32.cuh"
#include "qew_philox.cuh"
#include "qew_tune.cuh"

struct qew_langevin {
    qew_ctx *ctx = nullptr;
    int n = 0;
    uint64_t seed = 0;
    uint64_t step = 0;
    double *grad = nullptr;  // LangevinDynamics::grad_, dynamics.h:68
};

namespace {

constexpr int kBS = 256;

// dynamics.h:40-58 (diff > 0): one thread per site pair, one Philox block.
__global__ void k_langevin_update_rng(double *__restrict__ h, const double *__restrict__ grad,
                                      int n, double a, double b, uint64_t seed, uint64_t step) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i0 = 2 * j;
    if (i0 >= n) return;
    double z0, z1;
    philox_normal_pair(seed, step, (uint32_t)j, z0, z1);
    h[i0] += -a * grad[i0] + b * z0;
    if (i0 + 1 < n) h[i0 + 1] += -a * grad[i0 + 1] + b * z1;
}

// dynamics.h:59-62 (diff <= 0): pure gradient descent, no random numbers.
__global__ void k_langevin_update_det(double *__restrict__ h, const double *__restrict__ grad,
                                      int n, double a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) h[i] += -a * grad[i];
}

// Caller-supplied increments.
__global__ void k_langevin_update_xi(double *__restrict__ h, const double *__restrict__ grad,
                                     int n, double a, double b, const double *__restrict__ xi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) h[i] += -a * grad[i] + b * xi[i];
}

__global__ void k_philox_fill(double *out, int n, uint64_t seed, uint64_t step) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i0 = 2 * j;
    if (i0 >= n) return;
    double z0, z1;
    philox_normal_pair(seed, step, (uint32_t)j, z0, z1);
    out[i0] = z0;
    if (i0 + 1 < n) out[i0 + 1] = z1;
}

// ---- many steps in one cooperative persistent kernel ----
// The annealing loop of dynamic_anneal (qew_runs.h:162-175) on the device:
// step k uses drift[k], diff[k] and Philox step index rstep[k]. Heights are
// double-buffered (every gradient reads the previous step's line, as the
// reference's gradient-then-update does), one bounded grid barrier per step.
constexpr int kRunBS = 128;  // 64 measured the same, 32 slower (L = 65536)
constexpr int kRunTile = 2 * kRunBS;  // a thread owns one site pair (one Philox block)

// Box-Muller in FP32 from the same Philox block: 24-bit uniforms, FP32
// log / sqrt / sincospi (the FP32-gather run's increments).
__device__ __forceinline__ void philox_normal_pair_f32(uint64_t seed, uint64_t step, uint32_t j,
                                                       double &z0, double &z1) {
    uint32_t c[4] = {j, 0u, (uint32_t)step, (uint32_t)(step >> 32)};
    philox4x32_10(c, seed);
    const float u1 = ((float)(c[0] >> 8) + 1.0f) * (1.0f / 16777216.0f);
    const float u2 = (float)(c[2] >> 8) * (1.0f / 16777216.0f);
    const float r = sqrtf(-2.0f * logf(u1));
    float s, co;
    sincospif(2.0f * u2, &s, &co);
    z0 = (double)(r * co);
    z1 = (double)(r * s);
}

template <class Noise, bool NORMAL32>
__global__ void __launch_bounds__(kRunBS)
k_langevin_run(Noise nz, double *h, double *tmp, int n, LineDx L, double lt, double f, int model,
               int steps, const double *__restrict__ drift, const double *__restrict__ diff,
               const unsigned long long *__restrict__ rstep, uint64_t seed, GridSync *sync) {
    __shared__ double s_h[kRunTile + 2];
    __shared__ double s_dv[kRunTile + 1];
    __shared__ double s_sl[kRunTile + 1];
    const bool arc = (model == QEW_MODEL_ARCLENGTH);
    const int t = threadIdx.x;
    double *cur = h, *nxt = tmp;
    for (int k = 0; k < steps; ++k) {
        const double a = drift[k], b = diff[k];
        const uint64_t rs = rstep[k];
        for (int base = blockIdx.x * kRunTile; base < n; base += gridDim.x * kRunTile) {
            const int cnt = min(kRunTile, n - base);
            for (int j = t; j < cnt; j += kRunBS) s_h[j + 1] = __ldcg(cur + base + j);
            if (t == 0) s_h[0] = __ldcg(cur + (base == 0 ? n - 1 : base - 1));
            if (t == kRunBS - 1) s_h[cnt + 1] = __ldcg(cur + ((base + cnt == n) ? 0 : base + cnt));
            __syncthreads();
            for (int j = t; j < cnt; j += kRunBS)
                edge_gradient(nz, base + j, n, s_h[j + 1], s_h[j + 2], L, arc, s_dv[j + 1], s_sl[j + 1]);
            if (t == 0)
                edge_gradient(nz, base == 0 ? n - 1 : base - 1, n, s_h[0], s_h[1], L, arc, s_dv[0],
                              s_sl[0]);
            __syncthreads();
            const int j0 = 2 * t;
            if (j0 < cnt) {
                double z0 = 0.0, z1 = 0.0;
                if (b > 0) {
                    const uint32_t pair = (uint32_t)((base + j0) >> 1);
                    if (NORMAL32)
                        philox_normal_pair_f32(seed, rs, pair, z0, z1);
                    else
                        philox_normal_pair(seed, rs, pair, z0, z1);
                }
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int j = j0 + q;
                    if (j >= cnt) break;
                    const double g = site_gradient(s_h[j], s_h[j + 1], s_h[j + 2], s_dv[j],
                                                   s_dv[j + 1], s_sl[j], s_sl[j + 1], L, lt, f, arc);
                    const double z = q ? z1 : z0;
                    nxt[base + j] = (b > 0) ? s_h[j + 1] + (-a * g + b * z) : s_h[j + 1] + -a * g;
                }
            }
            __syncthreads();
        }
        if (!grid_sync_bounded(sync, gridDim.x)) return;
        double *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    if (cur != h)
        for (int i = blockIdx.x * kRunBS + t; i < n; i += gridDim.x * kRunBS) h[i] = __ldcg(cur + i);
}

// ---- the same run with K steps per grid barrier (temporal blocking) ----
// CTA b owns the segment [b*seg, b*seg + S) of the ring (S = seg, shorter or
// empty for the last CTAs). A round of Kr <= K steps loads the heights of
// [s0 - Kr, s0 + S + Kr) (periodic) into shared memory and advances them
// there: step s updates the positions s .. (region end - s) from step s - 1's
// values, so the segment's heights after Kr steps are exactly those of Kr
// single steps of the whole ring. Every position is computed as the one-step
// kernel computes it (the same edge and site functions on the same operands,
// the same increments: a site's Philox block is its global site pair's), so
// the results are bitwise those of k_langevin_run; the halo positions are
// computed by both neighbouring CTAs. One grid barrier per round.
//
// Shared memory, in doubles of the region R = seg + 2K: heights (two
// buffers), edge values, arclength slopes, increments.
constexpr int kTbBufs = 5;
// Dynamic shared memory a launch may take without raising the kernel's limit
// (48 KB less room for the kernel's static shared memory).
constexpr int kDefaultDynSmem = 47 * 1024;

template <class Noise, bool NORMAL32>
__global__ void __launch_bounds__(kRunBS)
k_langevin_run_tb(Noise nz, double *h, double *tmp, int n, LineDx L, double lt, double f,
                  int model, int steps, const double *__restrict__ drift,
                  const double *__restrict__ diff, const unsigned long long *__restrict__ rstep,
                  uint64_t seed, GridSync *sync, int seg, int K) {
    extern __shared__ double s_tb[];
    const int R = seg + 2 * K;
    double *hA = s_tb, *hB = s_tb + R, *dv = s_tb + 2 * R, *sl = s_tb + 3 * R,
           *zz = s_tb + 4 * R;
    const bool arc = (model == QEW_MODEL_ARCLENGTH);
    const int t = threadIdx.x;
    const int s0 = blockIdx.x * seg;
    const int S = max(0, min(seg, n - s0));
    double *cur = h, *nxt = tmp;
    for (int k0 = 0; k0 < steps; k0 += K) {
        const int Kr = min(K, steps - k0);
        if (S > 0) {
            // local position r <-> global site (s0 - Kr + r) mod n, r in [0, S + 2 Kr)
            int g0 = (s0 - Kr) % n;
            if (g0 < 0) g0 += n;
            auto gsite = [&](int r) {
                int g = g0 + r;
                if (g >= n) g -= n;
                if (g >= n) g %= n;  // a ring shorter than the region
                return g;
            };
            const int RS = S + 2 * Kr;
            for (int r = t; r < RS; r += kRunBS) hA[r] = __ldcg(cur + gsite(r));
            __syncthreads();
            for (int s = 1; s <= Kr; ++s) {
                const int k = k0 + s - 1;
                const double a = drift[k], b = diff[k];
                const uint64_t rs = rstep[k];
                const int lo = s, hi = RS - s;  // positions updated at this step
                for (int r = lo - 1 + t; r < hi; r += kRunBS)
                    edge_gradient(nz, gsite(r), n, hA[r], hA[r + 1], L, arc, dv[r], sl[r]);
                if (b > 0) {
                    for (int r = lo + t; r < hi; r += kRunBS) {
                        const int g = gsite(r);
                        if ((g & 1) && r != lo) continue;  // its pair's first site wrote it
                        double z0, z1;
                        if (NORMAL32)
                            philox_normal_pair_f32(seed, rs, (uint32_t)(g >> 1), z0, z1);
                        else
                            philox_normal_pair(seed, rs, (uint32_t)(g >> 1), z0, z1);
                        zz[r] = (g & 1) ? z1 : z0;
                        if (!(g & 1) && r + 1 < hi && g + 1 < n) zz[r + 1] = z1;
                    }
                }
                __syncthreads();
                for (int r = lo + t; r < hi; r += kRunBS) {
                    const double gr = site_gradient(hA[r - 1], hA[r], hA[r + 1], dv[r - 1], dv[r],
                                                    sl[r - 1], sl[r], L, lt, f, arc);
                    hB[r] = (b > 0) ? hA[r] + (-a * gr + b * zz[r]) : hA[r] + -a * gr;
                }
                __syncthreads();
                double *sw = hA;
                hA = hB;
                hB = sw;
            }
            for (int r = Kr + t; r < Kr + S; r += kRunBS) nxt[s0 + r - Kr] = hA[r];
        }
        if (!grid_sync_bounded(sync, gridDim.x)) return;
        double *sw = cur;
        cur = nxt;
        nxt = sw;
    }
    if (cur != h)
        for (int i = blockIdx.x * kRunBS + t; i < n; i += gridDim.x * kRunBS) h[i] = __ldcg(cur + i);
}

// Whether a functor gathers from the FP64 cell-polynomial store (a tuning class of its own).
template <class Noise>
bool reads_poly_store(const Noise &) { return false; }
bool reads_poly_store(const NoiseBSpline64 &nz) { return nz.poly != nullptr; }

qew_status check(qew_langevin *l, const qew_field *field, double *d_h, const qew_params *p) {
    if (!l || !l->ctx) return QEW_ERR_INVALID;
    if (!field || !d_h || !p)
        return qew_fail(l->ctx, QEW_ERR_INVALID, "langevin_step: bad arguments");
    return QEW_OK;
}

}  // namespace

extern "C" {

qew_status qew_langevin_create(qew_ctx *ctx, int n, uint64_t seed, qew_langevin **out) {
    if (!ctx || !out || n < 1) return qew_fail(ctx, QEW_ERR_INVALID, "langevin_create: bad arguments");
    qew_langevin *l = new (std::nothrow) qew_langevin();
    if (!l) return QEW_ERR_NOMEM;
    l->ctx = ctx;
    l->n = n;
    l->seed = seed;
    if (qew_alloc_async(ctx, (void **)&l->grad, sizeof(double) * (size_t)n) != QEW_OK) {
        delete l;
        return QEW_ERR_NOMEM;
    }
    *out = l;
    return QEW_OK;
}

qew_status qew_langevin_destroy(qew_langevin *l) {
    if (!l) return QEW_OK;
    if (l->grad) qew_free_async(l->grad, l->ctx->stream);
    delete l;
    return QEW_OK;
}

qew_status qew_langevin_step(qew_langevin *l, const qew_field *field, double *d_h,
                             const qew_params *p, double drift, double diff) {
    QEW_RANGE();
    QEW_TRY(check(l, field, d_h, p));
    qew_ctx *ctx = l->ctx;
    const int n = l->n;
    QEW_TRY(qew_gradient_enqueue(ctx, field, d_h, n, p, QEW_PREC_FP64, l->grad));
    if (diff > 0) {
        const int pairs = (n + 1) / 2;
        k_langevin_update_rng<<<(pairs + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(
            d_h, l->grad, n, drift, diff, l->seed, l->step);
        ++l->step;
    } else {
        k_langevin_update_det<<<(n + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(d_h, l->grad, n, drift);
    }
    return qew_launch_check(ctx, "langevin_update");
}

qew_status qew_langevin_step_increments(qew_langevin *l, const qew_field *field, double *d_h,
                                        const qew_params *p, double drift, double diff,
                                        const double *d_xi) {
    QEW_RANGE();
    QEW_TRY(check(l, field, d_h, p));
    qew_ctx *ctx = l->ctx;
    const int n = l->n;
    QEW_TRY(qew_gradient_enqueue(ctx, field, d_h, n, p, QEW_PREC_FP64, l->grad));
    if (diff > 0) {
        if (!d_xi) return qew_fail(ctx, QEW_ERR_INVALID, "langevin_step_increments: null xi");
        k_langevin_update_xi<<<(n + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(d_h, l->grad, n, drift,
                                                                          diff, d_xi);
    } else {
        k_langevin_update_det<<<(n + kBS - 1) / kBS, kBS, 0, ctx->stream>>>(d_h, l->grad, n, drift);
    }
    return qew_launch_check(ctx, "langevin_update");
}

qew_status qew_langevin_peek_increments(qew_langevin *l, double *d_xi) {
    if (!l || !l->ctx || !d_xi) return QEW_ERR_INVALID;
    const int pairs = (l->n + 1) / 2;
    k_philox_fill<<<(pairs + kBS - 1) / kBS, kBS, 0, l->ctx->stream>>>(d_xi, l->n, l->seed, l->step);
    return qew_launch_check(l->ctx, "philox_fill");
}

uint64_t qew_langevin_steps(const qew_langevin *l) { return l ? l->step : 0; }

qew_status qew_langevin_run(qew_langevin *l, const qew_field *field, double *d_h,
                            const qew_params *p, int steps, const double *h_drift,
                            const double *h_diff, int precision) {
    QEW_RANGE();
    QEW_TRY(check(l, field, d_h, p));
    qew_ctx *ctx = l->ctx;
    if (steps < 0 || (steps > 0 && (!h_drift || !h_diff)))
        return qew_fail(ctx, QEW_ERR_INVALID, "langevin_run: bad schedule");
    if (steps == 0) return QEW_OK;
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
    if (!coop) return qew_fail(ctx, QEW_ERR_UNSUPPORTED, "langevin_run: no cooperative launch");
    const int n = l->n;
    // Philox step index of each step: the counter advances on diff > 0 steps
    std::vector<unsigned long long> rs(steps);
    uint64_t c = l->step;
    for (int k = 0; k < steps; ++k) {
        rs[k] = c;
        if (h_diff[k] > 0) ++c;
    }
    const size_t vec = ((size_t)n * 8 + 255) & ~size_t(255);
    const size_t off_diff = ((size_t)steps * 8 + 255) & ~size_t(255);
    const size_t off_rs = off_diff + (((size_t)steps * 8 + 255) & ~size_t(255));
    const size_t off_tmp = off_rs + (((size_t)steps * 8 + 255) & ~size_t(255));
    const size_t off_probe = off_tmp + vec;   // the tuning probe's line and its buffer
    const size_t off_sync = off_probe + 2 * vec;
    QEW_TRY(qew_scratch_reserve(ctx, off_sync + sizeof(GridSync) + 256));
    char *base = (char *)ctx->scratch;
    double *d_drift = (double *)base, *d_diff = (double *)(base + off_diff);
    unsigned long long *d_rs = (unsigned long long *)(base + off_rs);
    double *tmp = (double *)(base + off_tmp);
    double *probe_h = (double *)(base + off_probe), *probe_tmp = probe_h + vec / 8;
    GridSync *sync = (GridSync *)(base + off_sync);
    QEW_CUDA(ctx, cudaMemcpyAsync(d_drift, h_drift, (size_t)steps * 8, cudaMemcpyHostToDevice, ctx->stream));
    QEW_CUDA(ctx, cudaMemcpyAsync(d_diff, h_diff, (size_t)steps * 8, cudaMemcpyHostToDevice, ctx->stream));
    QEW_CUDA(ctx, cudaMemcpyAsync(d_rs, rs.data(), (size_t)steps * 8, cudaMemcpyHostToDevice, ctx->stream));
    LineDx L = make_line_dx(p->physical_size, n);
    double lt = p->line_tension, fd = p->driving_force;
    int model = p->model;
    uint64_t seed = l->seed;
    int max_smem = 0;
    QEW_CUDA(ctx, cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                         ctx->device));
    // Candidates (bitwise-equal results): 0 = one grid barrier per step
    // (k_langevin_run); 1 + 3 i + j = temporal blocking at {1, 2, 4}[i] CTAs
    // per SM and K = {8, 16, 32}[j] steps per barrier.
    static const char *const names[10] = {
        "1 step per barrier", "K=8 x 1 CTA/SM", "K=16 x 1 CTA/SM", "K=32 x 1 CTA/SM",
        "K=8 x 2 CTA/SM", "K=16 x 2 CTA/SM", "K=32 x 2 CTA/SM", "K=8 x 4 CTA/SM",
        "K=16 x 4 CTA/SM", "K=32 x 4 CTA/SM"};
    auto launch = [&](auto nz, auto normal32) -> qew_status {
        constexpr bool kN32 = decltype(normal32)::value;
        auto kern = k_langevin_run<decltype(nz), kN32>;
        auto kern_tb = k_langevin_run_tb<decltype(nz), kN32>;
        const int cap = ctx->warp_cap > 0 ? std::max(1, ctx->warp_cap / (kRunBS / 32)) : INT_MAX;
        // grid, segment and shared memory of candidate c (c >= 1); false when
        // its shared memory or co-residency does not fit
        auto shape = [&](int c, int &grid, int &seg, int &K, size_t &smem) -> bool {
            const int cps = 1 << ((c - 1) / 3);
            K = 8 << ((c - 1) % 3);
            grid = std::min(std::min(ctx->num_sms * cps, cap), std::max(1, n / 64));
            seg = (n + grid - 1) / grid;
            grid = (n + seg - 1) / seg;  // no empty CTAs
            smem = (size_t)kTbBufs * (size_t)(seg + 2 * K) * sizeof(double);
            if (smem > (size_t)max_smem) return false;
            // Above the default 48 KB the kernel's dynamic shared-memory limit is
            // raised to this shape's size, never lowered: under a lock, from the
            // limit the device reports now (so a reset context is raised again),
            // so a launch on another host thread never finds it below its own.
            if (smem > (size_t)kDefaultDynSmem) {
                static std::mutex mu;
                std::lock_guard<std::mutex> lock(mu);
                cudaFuncAttributes fa{};
                if (cudaFuncGetAttributes(&fa, (const void *)kern_tb) != cudaSuccess) {
                    cudaGetLastError();
                    return false;
                }
                if (fa.maxDynamicSharedSizeBytes < (int)smem &&
                    cudaFuncSetAttribute((const void *)kern_tb,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem) != cudaSuccess) {
                    cudaGetLastError();
                    return false;
                }
            }
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern_tb, kRunBS, smem) !=
                cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            return grid <= per_sm * ctx->num_sms;
        };
        // candidate c on line hh (buffer tt) for nsteps steps of the schedule
        auto run_on = [&](int c, double *hh, double *tt, int nsteps) -> qew_status {
            QEW_TRY(qew_gridsync_init(ctx, sync));
            int grid, seg, K;
            size_t smem;
            if (c >= 1 && shape(c, grid, seg, K, smem)) {
                void *args[] = {(void *)&nz,     (void *)&hh,     (void *)&tt,     (void *)&n,
                                (void *)&L,      (void *)&lt,     (void *)&fd,     (void *)&model,
                                (void *)&nsteps, (void *)&d_drift, (void *)&d_diff, (void *)&d_rs,
                                (void *)&seed,   (void *)&sync,   (void *)&seg,    (void *)&K};
                QEW_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)kern_tb, dim3(grid),
                                                          dim3(kRunBS), args, smem, ctx->stream));
                return qew_launch_check(ctx, "langevin_run");
            }
            int per_sm = 0;
            QEW_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRunBS, 0));
            const int want = (n + kRunTile - 1) / kRunTile;
            const int slots = std::min(ctx->num_sms * std::max(per_sm, 1), cap);
            const int g1 = std::max(1, std::min(want, slots));
            void *args[] = {(void *)&nz,     (void *)&hh,      (void *)&tt,     (void *)&n,
                            (void *)&L,      (void *)&lt,      (void *)&fd,     (void *)&model,
                            (void *)&nsteps, (void *)&d_drift, (void *)&d_diff, (void *)&d_rs,
                            (void *)&seed,   (void *)&sync};
            QEW_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)kern, dim3(g1), dim3(kRunBS),
                                                      args, 0, ctx->stream));
            return qew_launch_check(ctx, "langevin_run");
        };
        // Runs of at least kTuneSteps steps time the candidates on a copy of
        // the line (64 steps each, the schedule's first); shorter runs take a
        // choice already made for their class, else the default.
        constexpr int kTuneSteps = 4096, kProbeSteps = 64;
        const int cls = qew_tune_class(n, (kN32 ? 1 : 0) + (model == QEW_MODEL_ARCLENGTH ? 2 : 0) +
                                              (reads_poly_store(nz) ? 4 : 0));
        // Defaults from measurement at L = 65536: FP32 runs K = 16 steps per
        // barrier at 2 CTAs per SM (515 against 804 us per 64 steps); FP64
        // runs one barrier per step, where the FP64 work of a step (the FP64
        // Box-Muller increments above all) outweighs the barrier and the
        // halo's extra work made the blocked shapes no faster. A tuned shape
        // must be 5 % faster than the default on the probe.
        const int dflt = kN32 ? 5 : 0;
        int cand = dflt;
        const int cached = qew_tune_cached(ctx->device, kTuneLangevinRun, cls);
        if (ctx->tune_force[kTuneLangevinRun] >= 0 || (cached < 0 && steps >= kTuneSteps)) {
            auto probe = [&](int c) -> qew_status {
                QEW_CUDA(ctx, cudaMemcpyAsync(probe_h, d_h, (size_t)n * 8,
                                              cudaMemcpyDeviceToDevice, ctx->stream));
                return run_on(c, probe_h, probe_tmp, kProbeSteps);
            };
            QEW_TRY(qew_tune_pick(ctx, kTuneLangevinRun, cls, 10, dflt, names, probe, &cand,
                                  0.05f));
        } else if (cached >= 0 && ctx->autotune) {
            cand = cached;
        } else if (!ctx->autotune) {
            cand = dflt;
        }
        return run_on(cand, d_h, tmp, steps);
    };
    if (precision == QEW_PREC_FP32_SPLIT) {
        if (field->kind != QEW_FIELD_BSPLINE || !field->coef32)
            return qew_fail(ctx, QEW_ERR_INVALID, "langevin_run: FP32 gather needs QEW_STORE_FP32");
        QEW_TRY(launch(make_split32(field, n, p->physical_size), std::true_type{}));
    } else {
        QEW_TRY(qew_dispatch_noise(ctx, field, [&](auto nz) {
            return launch(nz, std::false_type{});
        }, n, p->physical_size));
    }
    GridSync hs;
    QEW_CUDA(ctx, cudaMemcpyAsync(&hs, sync, sizeof(GridSync), cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hs.err) return qew_fail(ctx, QEW_ERR_TIMEOUT, "langevin_run: grid barrier timed out");
    l->step = c;
    return QEW_OK;
}

}  // extern "C"
