// qew_lbfgs_resident.cu -- device-resident L-BFGS: the whole lbfgs_minimize
// (lbfgs.h:94-287) of one line runs inside one CTA, with every reduction a
// CTA reduction and every scalar decision (Armijo test, curvature skip,
// history ring, restarts) taken on the device. One launch per solve instead
// of ~4m+10 launches and ~2m+4 device->host reads per iteration.
//
// Control flow, defaults and result fields are those of the reference; the
// arithmetic differs only in reduction order (CTA trees instead of a serial
// sum) and in the preconditioner, applied as the exact factorised periodic
// solve (qew_block.cuh) instead of rfft / divide / irfft.
//
// A long line is solved by a thread-block cluster instead of one CTA: the
// FP64 work of each iteration (gathers, dot products) spreads over up to 16
// SMs, reductions go through distributed shared memory and the barriers are
// cluster barriers (qew_team.cuh). Lines of at least kClusterMinN points take
// this form; the arithmetic differs from the one-CTA form only in the
// reduction order.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "qew_lbfgs_internal.cuh"
#include "qew_noise32.cuh"
#include "qew_lbfgs_resident.cuh"

PrecondCoef qew_precond_coef(int n, double kappa, double physical_size, double shift) {
    PrecondCoef pc{};
    const double dx = physical_size / (double)n;
    const double sigma = qew_precond_shift_rule(n, kappa, physical_size, shift);
    const double a = kappa / dx;
    if (!(a > 0)) {
        pc.scalar = 1;
        pc.inv_sigma = 1.0 / sigma;
        return pc;
    }
    const double e = sigma / (2.0 * a);
    const double zm1 = e - std::sqrt(e * (2.0 + e));  // z - 1, no cancellation
    pc.z = 1.0 + zm1;
    pc.logz = std::log1p(zm1);
    pc.inv_1mzn = -1.0 / std::expm1((double)n * pc.logz);
    pc.gain = pc.z / a;
    pc.scalar = 0;
    return pc;
}

namespace {

constexpr int kResBS = 512;

template <int BS>
__global__ void __launch_bounds__(BS) k_precond_resident(const double *q, double *d, int n,
                                                         PrecondCoef pc) {
    __shared__ double s_b[BS];
    __shared__ double s_w[96];
    block_precond<BS>(q, d, n, pc, s_b, s_w);
}

constexpr int kClusterBS = 256;
constexpr int kClusterMinN = 2048;
#ifndef QEW_CLUSTER_POINTS_PER_THREAD
#define QEW_CLUSTER_POINTS_PER_THREAD 1  // build-time tuning knob (measured on GB300)
#endif

// One line of a cluster launch (all lines of a launch share n and the field).
struct ClusterLine {
    double *h;
    qew_params p;
    PrecondCoef pc;
};

template <class Noise, int BS>
__global__ void __launch_bounds__(BS)
k_lbfgs_cluster(Noise nz, const ClusterLine *__restrict__ lines, int n, LbfgsCfg cfg, double *ws,
                size_t ws_stride, size_t npad, qew_lbfgs_result *out) {
    __shared__ double s_w[96];
    __shared__ double s_red[2 * 3 * kTeamMaxCtas];
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    const unsigned size = cl.num_blocks();
    ClusterTeam<BS> T{s_w, s_red, cl.block_rank(), size};
    const int line = blockIdx.x / size;
    const ClusterLine L = lines[line];
    const qew_lbfgs_result r =
        lbfgs_team<Noise>(T, nz, L.h, n, L.p, cfg, L.pc, ws + (size_t)line * ws_stride, npad);
    if (T.rank() == 0 && threadIdx.x == 0) out[line] = r;
    cl.sync();  // no CTA leaves while another may still write its shared memory
}

template <class Noise, int BS>
__global__ void __launch_bounds__(BS)
k_lbfgs_single(Noise nz, double *h, int n, qew_params P, LbfgsCfg cfg, PrecondCoef pc,
               double *ws, size_t npad, qew_lbfgs_result *out) {
    extern __shared__ double s_dyn[];
    const qew_lbfgs_result r = lbfgs_block<Noise, BS>(nz, h, n, P, cfg, pc, ws, npad);
    if (threadIdx.x == 0) *out = r;
}

}  // namespace

// Cluster size for a line of n points: about QEW_CLUSTER_POINTS_PER_THREAD
// points per thread, a power of two between 4 and 16 CTAs, 0 when the line is
// too short or the device cannot co-schedule such a cluster (the one-CTA
// form is used then).
template <class Noise>
static int cluster_size_for(qew_ctx *ctx, int n) {
    if (n < kClusterMinN) return 0;
    int c = 1;
    while (c < kTeamMaxCtas &&
           (long long)c * 2 * kClusterBS * QEW_CLUSTER_POINTS_PER_THREAD <= n)
        c *= 2;
    if (c < 4) return 0;
    auto kern = k_lbfgs_cluster<Noise, kClusterBS>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        c = std::min(c, 8);
    }
    for (; c >= 4; c /= 2) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(c);
        lc.blockDim = dim3(kClusterBS);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = c;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, kern, &lc) == cudaSuccess && clusters > 0)
            return c;
        cudaGetLastError();
    }
    (void)ctx;
    return 0;
}

// Relaxes `count` lines of n points (device pointers in lines[k].h) on one
// field, one cluster of `csize` CTAs per line.
template <class Noise>
static qew_status lbfgs_cluster_launch(qew_ctx *ctx, const Noise &nz, int csize,
                                       const std::vector<ClusterLine> &lines, int n,
                                       const qew_lbfgs_params *lp, qew_lbfgs_result *res) {
    const int count = (int)lines.size();
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    const size_t wsd = qew_lbfgs_resident_ws_doubles(n, lp->m);
    const size_t off_lines = (wsd * count * sizeof(double) + 255) & ~size_t(255);
    const size_t off_res = (off_lines + sizeof(ClusterLine) * count + 255) & ~size_t(255);
    QEW_TRY(qew_scratch_reserve(ctx, off_res + sizeof(qew_lbfgs_result) * count + 256));
    char *base = (char *)ctx->scratch;
    ClusterLine *d_lines = (ClusterLine *)(base + off_lines);
    qew_lbfgs_result *d_res = (qew_lbfgs_result *)(base + off_res);
    QEW_CUDA(ctx, cudaMemcpyAsync(d_lines, lines.data(), sizeof(ClusterLine) * count,
                                  cudaMemcpyHostToDevice, ctx->stream));
    const LbfgsCfg cfg = lbfgs_cfg_from(lp);
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(count * csize));
    lc.blockDim = dim3(kClusterBS);
    lc.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    double *ws = (double *)base;
    QEW_CUDA(ctx, cudaLaunchKernelEx(&lc, k_lbfgs_cluster<Noise, kClusterBS>, nz,
                                     (const ClusterLine *)d_lines, n, cfg, ws, wsd, npad, d_res));
    QEW_TRY(qew_launch_check(ctx, "lbfgs_cluster"));
    QEW_CUDA(ctx, cudaMemcpyAsync(res, d_res, sizeof(qew_lbfgs_result) * count,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

size_t qew_lbfgs_resident_ws_doubles(int n, int m) {
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    return npad * (size_t)(kLbfgsVecs + 2 * (m + 1));
}

qew_status qew_lbfgs_resident(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                              const qew_params *p, const qew_lbfgs_params *lp,
                              qew_lbfgs_result *res) {
    if (lp->m > kLbfgsMaxM)
        return qew_fail(ctx, QEW_ERR_UNSUPPORTED, "lbfgs resident: m=%d exceeds %d", lp->m,
                        kLbfgsMaxM);
    PrecondCoef pc1{};
    if (lp->precondition) pc1 = qew_precond_coef(n, p->line_tension, p->physical_size, lp->precond_shift);
    bool clustered = false;
    QEW_TRY(qew_dispatch_noise(ctx, field, [&](auto nz) -> qew_status {
        const int csize = cluster_size_for<decltype(nz)>(ctx, n);
        if (!csize) return QEW_OK;
        clustered = true;
        return lbfgs_cluster_launch(ctx, nz, csize, std::vector<ClusterLine>{{d_h, *p, pc1}}, n, lp,
                                    res);
    }, n, p->physical_size));
    if (clustered) return QEW_OK;
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    const size_t wsd = qew_lbfgs_resident_ws_doubles(n, lp->m);
    const size_t res_off = (wsd * sizeof(double) + 255) & ~size_t(255);
    QEW_TRY(qew_scratch_reserve(ctx, res_off + sizeof(qew_lbfgs_result) + 256));
    double *ws = (double *)ctx->scratch;
    qew_lbfgs_result *d_res = (qew_lbfgs_result *)((char *)ctx->scratch + res_off);
    LbfgsCfg cfg = lbfgs_cfg_from(lp);
    PrecondCoef pc{};
    if (lp->precondition) pc = qew_precond_coef(n, p->line_tension, p->physical_size, lp->precond_shift);
    const size_t smem = lbfgs_block_smem_bytes(kResBS, lp->m);
    QEW_TRY(qew_dispatch_noise(ctx, field, [&](auto nz) -> qew_status {
        auto kern = k_lbfgs_single<decltype(nz), kResBS>;
        QEW_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<1, kResBS, smem, ctx->stream>>>(nz, d_h, n, *p, cfg, pc, ws, npad, d_res);
        return qew_launch_check(ctx, "lbfgs_resident");
    }, n, p->physical_size));
    QEW_CUDA(ctx, cudaMemcpyAsync(res, d_res, sizeof(qew_lbfgs_result), cudaMemcpyDeviceToHost, ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

qew_status qew_lbfgs_cluster_lines(qew_ctx *ctx, const qew_field *field, int count,
                                   double *const *d_h, int n, const qew_params *ps,
                                   const double *shifts, const qew_lbfgs_params *lp,
                                   qew_lbfgs_result *res, int precision) {
    if (count < 1 || lp->m > kLbfgsMaxM) return QEW_ERR_UNSUPPORTED;
    // one noise functor serves every line: they must share the x geometry
    for (int k = 1; k < count; ++k)
        if (ps[k].physical_size != ps[0].physical_size) return QEW_ERR_UNSUPPORTED;
    std::vector<ClusterLine> lines(count);
    for (int k = 0; k < count; ++k) {
        lines[k].h = d_h[k];
        lines[k].p = ps[k];
        lines[k].pc = lp->precondition ? qew_precond_coef(n, ps[k].line_tension, ps[k].physical_size,
                                                          shifts[k])
                                       : PrecondCoef{};
    }
    bool clustered = false;
    auto run = [&](auto nz) -> qew_status {
        const int csize = cluster_size_for<decltype(nz)>(ctx, n);
        if (!csize) return QEW_OK;
        clustered = true;
        return lbfgs_cluster_launch(ctx, nz, csize, lines, n, lp, res);
    };
    if (precision == QEW_PREC_FP32_SPLIT) {
        if (field->kind != QEW_FIELD_BSPLINE || !field->coef32) return QEW_ERR_UNSUPPORTED;
        QEW_TRY(run(make_split32(field, n, ps[0].physical_size)));
    } else {
        QEW_TRY(qew_dispatch_noise(ctx, field, run, n, ps[0].physical_size));
    }
    return clustered ? QEW_OK : QEW_ERR_UNSUPPORTED;
}

qew_status qew_precond_resident(qew_ctx *ctx, const double *d_q, int n, double kappa,
                                double physical_size, double shift, double *d_out) {
    const PrecondCoef pc = qew_precond_coef(n, kappa, physical_size, shift);
    k_precond_resident<kResBS><<<1, kResBS, 0, ctx->stream>>>(d_q, d_out, n, pc);
    QEW_TRY(qew_launch_check(ctx, "precond_resident"));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}
