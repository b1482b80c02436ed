// qew_langevin.cu -- overdamped Langevin / Euler-Maruyama step
// (LangevinDynamics, dynamics.h:27-70): h_i += -drift * dE/dh_i + diff * xi_i.
//
// The reference draws xi from Kokkos' Random_XorShift64_Pool, whose stream is
// specific to that library; here xi comes from a Philox4x32-10 counter stream
// keyed by (seed, site pair, step), so any step of any site can be regenerated
// independently (and by the oracle, bit-for-bit in the uniforms). Trajectory
// parity with the reference is checked through the increments entry point,
// which takes xi from the caller.
#include <new>

#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"
#include "qew_philox.cuh"

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
    if (cudaMalloc(&l->grad, sizeof(double) * (size_t)n) != cudaSuccess) {
        cudaGetLastError();
        delete l;
        return qew_fail(ctx, QEW_ERR_NOMEM, "langevin_create: cudaMalloc");
    }
    *out = l;
    return QEW_OK;
}

qew_status qew_langevin_destroy(qew_langevin *l) {
    if (!l) return QEW_OK;
    if (l->grad) {
        cudaStreamSynchronize(l->ctx->stream);
        cudaFree(l->grad);
    }
    delete l;
    return QEW_OK;
}

qew_status qew_langevin_step(qew_langevin *l, const qew_field *field, double *d_h,
                             const qew_params *p, double drift, double diff) {
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

}  // extern "C"
