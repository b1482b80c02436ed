// qew_fire.cu -- fire_minimize (fire.h:41-131): FIRE relaxation (Bitzek et
// al., PRL 97, 170201 (2006)), semi-implicit Euler variant, as one kernel with
// one CTA per line. The reference runs each vector operation and reduction as
// its own parallel dispatch with a host round trip; here the whole loop --
// gradient, max|g| test, velocity step, power, mixing, position step -- stays
// in the CTA, with deterministic CTA reductions (warp butterflies, warp
// partials added in warp order), so a run is reproducible bit for bit.
#include "qew_block.cuh"

namespace {

constexpr int kFireBS = 512;

struct FireCfg {
    double dt_max, dt_init, ftol;
    int max_iter, n_min;
    double f_inc, f_dec, alpha_start, f_alpha;
};

template <class Noise, int BS>
__global__ void __launch_bounds__(BS)
k_fire(Noise nz, double *__restrict__ h, int n, qew_params P, FireCfg c, double *ws, size_t npad,
       qew_fire_result *out) {
    __shared__ double s_w[96];
    double *g = ws, *v = ws + npad, *ev = ws + 2 * npad, *es = ws + 3 * npad;
    const LineDx dx = make_line_dx(P.physical_size, n);
    const bool arc = (P.model == QEW_MODEL_ARCLENGTH);
    const double lt = P.line_tension, fd = P.driving_force;
    for (int i = threadIdx.x; i < n; i += BS) v[i] = 0.0;
    double dt = (c.dt_init > 0) ? c.dt_init : 0.1 * c.dt_max;
    double alpha = c.alpha_start;
    int n_pos = 0;
    block_gradient<Noise, BS>(nz, h, n, dx, lt, fd, arc, ev, es, g);
    qew_fire_result res{};
    for (int it = 0; it < c.max_iter; ++it) {
        double m = 0.0;
        for (int i = threadIdx.x; i < n; i += BS) m = fmax(m, fabs(g[i]));
        m = bmax_all<BS>(m, s_w);
        if (m < c.ftol) {
            res.iterations = it;
            res.max_force = m;
            res.converged = 1;
            if (threadIdx.x == 0) *out = res;
            return;
        }
        // v += dt F (F = -grad), then the power P = F . v
        double pw = 0.0;
        for (int i = threadIdx.x; i < n; i += BS) {
            const double vi = v[i] - dt * g[i];
            v[i] = vi;
            pw += -g[i] * vi;
        }
        pw = bsum_all<BS>(pw, s_w);
        if (pw > 0) {
            if (n_pos > c.n_min) {
                dt = fmin(dt * c.f_inc, c.dt_max);
                alpha *= c.f_alpha;
            }
            ++n_pos;
        } else {
            for (int i = threadIdx.x; i < n; i += BS) v[i] = 0.0;
            dt *= c.f_dec;
            alpha = c.alpha_start;
            n_pos = 0;
        }
        // mix v toward F: v = (1 - a) v + a |v| / |F| F
        double nv2 = 0.0, nf2 = 0.0, unused = 0.0;
        for (int i = threadIdx.x; i < n; i += BS) {
            nv2 += v[i] * v[i];
            nf2 += g[i] * g[i];
        }
        bsum3_all<BS>(nv2, nf2, unused, s_w);
        const double nf = sqrt(nf2);
        if (nf > 0) {
            const double a = alpha;
            const double scale = alpha * sqrt(nv2) / nf;
            for (int i = threadIdx.x; i < n; i += BS) v[i] = (1.0 - a) * v[i] - scale * g[i];
        }
        for (int i = threadIdx.x; i < n; i += BS) h[i] += dt * v[i];
        __syncthreads();  // the gradient reads neighbours written by other threads
        block_gradient<Noise, BS>(nz, h, n, dx, lt, fd, arc, ev, es, g);
    }
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += BS) m = fmax(m, fabs(g[i]));
    m = bmax_all<BS>(m, s_w);
    res.iterations = c.max_iter;
    res.max_force = m;
    res.converged = 0;
    if (threadIdx.x == 0) *out = res;
}

}  // namespace

extern "C" {

qew_status qew_fire_default_params(qew_fire_params *fp) {
    if (!fp) return QEW_ERR_INVALID;
    // FireParams, fire.h:21-31
    fp->dt_max = 0.0;
    fp->dt_init = 0.0;
    fp->ftol = 1e-6;
    fp->max_iter = 100000;
    fp->n_min = 5;
    fp->f_inc = 1.1;
    fp->f_dec = 0.5;
    fp->alpha_start = 0.1;
    fp->f_alpha = 0.99;
    return QEW_OK;
}

qew_status qew_fire_minimize(qew_ctx *ctx, const qew_field *field, double *d_h, int n,
                             const qew_params *p, const qew_fire_params *fp,
                             qew_fire_result *res) {
    QEW_RANGE();
    if (!ctx || !field || !d_h || !p || !fp || !res || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "fire_minimize: bad arguments");
    if (!(fp->dt_max > 0) || fp->max_iter < 0)
        return qew_fail(ctx, QEW_ERR_INVALID, "fire_minimize: dt_max must be > 0");
    QEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t npad = ((size_t)n + 31) & ~size_t(31);
    const size_t res_off = (4 * npad * sizeof(double) + 255) & ~size_t(255);
    QEW_TRY(qew_scratch_reserve(ctx, res_off + sizeof(qew_fire_result) + 256));
    double *ws = (double *)ctx->scratch;
    qew_fire_result *d_res = (qew_fire_result *)((char *)ctx->scratch + res_off);
    const FireCfg c{fp->dt_max, fp->dt_init, fp->ftol, fp->max_iter, fp->n_min,
                    fp->f_inc, fp->f_dec, fp->alpha_start, fp->f_alpha};
    QEW_TRY(qew_dispatch_noise(ctx, field, [&](auto nz) -> qew_status {
        k_fire<decltype(nz), kFireBS><<<1, kFireBS, 0, ctx->stream>>>(nz, d_h, n, *p, c, ws, npad,
                                                                       d_res);
        return qew_launch_check(ctx, "fire");
    }, n, p->physical_size));
    QEW_CUDA(ctx, cudaMemcpyAsync(res, d_res, sizeof(qew_fire_result), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    QEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return QEW_OK;
}

}  // extern "C"
