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
#include <cmath>

#include "qew_block.cuh"
#include "qew_lbfgs_internal.cuh"
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

template <class Noise, int BS>
__global__ void __launch_bounds__(BS)
k_lbfgs_single(Noise nz, double *h, int n, qew_params P, LbfgsCfg cfg, PrecondCoef pc,
               double *ws, size_t npad, qew_lbfgs_result *out) {
    extern __shared__ double s_dyn[];
    const qew_lbfgs_result r = lbfgs_block<Noise, BS>(nz, h, n, P, cfg, pc, ws, npad);
    if (threadIdx.x == 0) *out = r;
}

}  // namespace

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

qew_status qew_precond_resident(qew_ctx *ctx, const double *d_q, int n, double kappa,
                                double physical_size, double shift, double *d_out) {
    const PrecondCoef pc = qew_precond_coef(n, kappa, physical_size, shift);
    k_precond_resident<kResBS><<<1, kResBS, 0, ctx->stream>>>(d_q, d_out, n, pc);
    QEW_TRY(qew_launch_check(ctx, "precond_resident"));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}
