// qew_block.cuh -- CTA-wide building blocks of the device-resident solvers:
// broadcast reductions, the model evaluated by one CTA over a whole line, and
// the periodic preconditioner solve.
#pragma once

#include "qew_internal.cuh"
#include "qew_lbfgs_internal.cuh"
#include "qew_model_kernels.cuh"

// Sum over the CTA, returned to every thread. Deterministic: warp butterfly,
// then every thread adds the warp partials in warp order.
template <int BS>
__device__ __forceinline__ double bsum_all(double v, double *s_w) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
#pragma unroll
    for (int k = 0; k < BS / 32; ++k) r += s_w[k];
    __syncthreads();
    return r;
}

template <int BS>
__device__ __forceinline__ double bmax_all(double v, double *s_w) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
#pragma unroll
    for (int k = 0; k < BS / 32; ++k) r = fmax(r, s_w[k]);
    __syncthreads();
    return r;
}

// Three sums at once (one pair of barriers).
template <int BS>
__device__ __forceinline__ void bsum3_all(double &a, double &b, double &c, double *s_w) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_w[w] = a;
        s_w[32 + w] = b;
        s_w[64 + w] = c;
    }
    __syncthreads();
    a = b = c = 0.0;
#pragma unroll
    for (int k = 0; k < BS / 32; ++k) {
        a += s_w[k];
        b += s_w[32 + k];
        c += s_w[64 + k];
    }
    __syncthreads();
}

// gradient() of a whole line by one CTA (qew_model.h:149-193): edge pass into
// ev/es, barrier, site combine into g. Ends with a barrier.
template <class Noise, int BS>
__device__ void block_gradient(const Noise &nz, const double *__restrict__ h, int n,
                               const LineDx &dx, double lt, double f, bool arc, double *ev,
                               double *es, double *g) {
    for (int e = threadIdx.x; e < n; e += BS) {
        const int ep = (e + 1 == n) ? 0 : e + 1;
        double dv, sl;
        edge_gradient(nz, e, n, h[e], h[ep], dx, arc, dv, sl);
        ev[e] = dv;
        es[e] = sl;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += BS) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const int im = (i == 0) ? n - 1 : i - 1;
        g[i] = site_gradient(h[im], h[i], h[ip], ev[im], ev[i], es[im], es[i], dx, lt, f, arc);
    }
    __syncthreads();
}

// objective() at x0 + alpha*d (alpha = 0: at x0) by one CTA.
template <class Noise, int BS>
__device__ double block_objective(const Noise &nz, const double *__restrict__ x0,
                                  const double *__restrict__ d, double alpha, int n,
                                  const LineDx &dx, double lt, double f, int model, double *s_w) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += BS) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const double hi = x0[i] + alpha * d[i];
        const double hip = x0[ip] + alpha * d[ip];
        acc += edge_energy(nz, i, ip, hi, hip, dx, lt, f, model);
    }
    return bsum_all<BS>(acc, s_w);
}

// y_k = x_k + z y_{k-1} on a periodic sequence of n values (index map
// k -> rev ? n-1-k : k), by one CTA: per-thread contiguous chunks, a CTA scan
// of the affine chunk maps (A, B) with A = z^len, B = zero-start chunk end,
// the periodic closure y_{-1} = Y_end / (1 - z^n), then a second chunk pass
// from the exact start values. In-place (out == in) is allowed. s_b needs BS
// doubles, s_w 2*(BS/32). Ends with a barrier.
template <int BS, class R = double>
__device__ void block_periodic_recurrence(const R *in, R *out, int n, bool rev,
                                          const PrecondCoef &pc, double *s_b, double *s_w) {
    const int t = threadIdx.x;
    const int c = (n + BS - 1) / BS;
    const int start = min(t * c, n);
    const int end = min(start + c, n);
    const double z = pc.z;
    double B = 0.0;
    for (int k = start; k < end; ++k) B = (double)in[rev ? n - 1 - k : k] + z * B;
    double A = (end > start) ? exp((double)(end - start) * pc.logz) : 1.0;
    // inclusive warp scan of (A, B), later element applied last
    const int lane = t & 31, w = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double Ap = __shfl_up_sync(0xffffffffu, A, o);
        const double Bp = __shfl_up_sync(0xffffffffu, B, o);
        if (lane >= o) {
            B = A * Bp + B;
            A = A * Ap;
        }
    }
    if (lane == 31) {
        s_w[w] = A;
        s_w[32 + w] = B;
    }
    __syncthreads();
    if (w == 0) {  // scan of warp aggregates
        double Aw = (lane < BS / 32) ? s_w[lane] : 1.0;
        double Bw = (lane < BS / 32) ? s_w[32 + lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double Ap = __shfl_up_sync(0xffffffffu, Aw, o);
            const double Bp = __shfl_up_sync(0xffffffffu, Bw, o);
            if (lane >= o) {
                Bw = Aw * Bp + Bw;
                Aw = Aw * Ap;
            }
        }
        if (lane < BS / 32) {
            s_w[lane] = Aw;
            s_w[32 + lane] = Bw;
        }
    }
    __syncthreads();
    if (w > 0) {  // prepend the previous warps' aggregate
        B = A * s_w[32 + w - 1] + B;
    }
    s_b[t] = B;  // inclusive zero-start value at the end of this chunk
    __syncthreads();
    const double y_end = s_b[BS - 1];
    const double P = y_end * pc.inv_1mzn;  // periodic y_{-1}
    const double cin = (t > 0) ? s_b[t - 1] : 0.0;
    const double E = cin + exp((double)start * pc.logz) * P;
    double y = E;
    for (int k = start; k < end; ++k) {
        const int idx = rev ? n - 1 - k : k;
        y = (double)in[idx] + z * y;
        out[idx] = (R)y;
    }
    __syncthreads();
}

// d = M^{-1} q (lbfgs.h:173-180) as the factorised periodic solve (vectors of
// R, arithmetic in FP64).
template <int BS, class R = double>
__device__ void block_precond(const R *q, R *d, int n, const PrecondCoef &pc, double *s_b,
                              double *s_w) {
    if (pc.scalar) {
        for (int i = threadIdx.x; i < n; i += BS) d[i] = (R)((double)q[i] * pc.inv_sigma);
        __syncthreads();
        return;
    }
    block_periodic_recurrence<BS, R>(q, d, n, false, pc, s_b, s_w);
    block_periodic_recurrence<BS, R>(d, d, n, true, pc, s_b, s_w);
    for (int i = threadIdx.x; i < n; i += BS) d[i] = (R)((double)d[i] * pc.gain);
    __syncthreads();
}
