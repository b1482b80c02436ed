// qew_model_kernels.cuh -- device kernels of the model layer, shared by the
// model entry points and the solvers (L-BFGS, Langevin).
#pragma once

#include "qew_internal.cuh"

// Line-position accessors of detail::objective_eval (qew_model.h:88-98).
struct LineAt {
    const double *__restrict__ h;
    __device__ __forceinline__ double operator()(int i) const { return h[i]; }
};
struct TrialAt {  // x0 + alpha*d, never materialised (qew_model.h:92-98)
    const double *__restrict__ x0;
    const double *__restrict__ d;
    double alpha;
    __device__ __forceinline__ double operator()(int i) const { return x0[i] + alpha * d[i]; }
};

// Energy of edge (i, ip): dx*(e_el + V(xc, hc) - f*h_i), qew_model.h:61-83.
template <class Noise>
__device__ __forceinline__ double edge_energy(const Noise &nz, int i, int ip, double hi,
                                              double hip, const LineDx &L, double lt, double f,
                                              int model) {
    // Unfused where a contraction would change the rounding (1 + s^2, the
    // f*h term), so the reference-exact functor reproduces its operations.
    const double dh_dx = L.div(hip - hi);
    double line_energy;
    if (model == QEW_MODEL_LINEAR)
        line_energy = lt * dh_dx * dh_dx * 0.5;
    else
        line_energy = lt * (sqrt(__dadd_rn(1.0, __dmul_rn(dh_dx, dh_dx))) - 1.0);
    const double xc = (double)(i + ip) * 0.5 * L.dx;
    const double hc = (hip + hi) * 0.5;
    return L.dx * __dsub_rn(__dadd_rn(line_energy, noise_value_edge(nz, i, xc, hc)),
                            __dmul_rn(f, hi));
}

// Edge pass of gradient(), qew_model.h:163-175: dV/dy at the midpoint of edge
// (e, e+1) and, for arclength, the normalised slope dh/sqrt(1+dh^2).
template <class Noise>
__device__ __forceinline__ void edge_gradient(const Noise &nz, int e, int n, double he,
                                              double hep, const LineDx &L, bool arc, double &dv,
                                              double &sl) {
    const int ep = (e + 1 == n) ? 0 : e + 1;
    const double xc = (double)(e + ep) * 0.5 * L.dx;
    const double hc = (hep + he) * 0.5;
    dv = noise_dvdy_edge(nz, e, xc, hc);
    sl = 0.0;
    if (arc) {
        const double dh = L.div(hep - he);
        sl = dh / sqrt(__dadd_rn(1.0, __dmul_rn(dh, dh)));
    }
}

// Per-site combine, qew_model.h:177-193.
__device__ __forceinline__ double site_gradient(double hm, double h0, double hp, double dvl,
                                                double dvr, double sll, double slr,
                                                const LineDx &L, double lt, double f, bool arc) {
    double line_force;
    if (!arc) {
        const double d2h = hm + hp - 2.0 * h0;
        line_force = L.div2(-lt * d2h);
    } else {
        line_force = L.div(lt * (sll - slr));
    }
    return L.dx * (line_force + 0.5 * (dvl + dvr) - f);
}

// Fused gradient: CTA of BS sites stages h[base-1 .. base+BS] and the BS+1
// edges it needs (its own plus the left halo edge) in shared memory.
template <class Noise, int BS>
__global__ void __launch_bounds__(BS)
k_gradient(const double *__restrict__ h, int n, LineDx dx, double lt, double f, int model,
           Noise nz, double *__restrict__ grad) {
    __shared__ double s_h[BS + 2];
    __shared__ double s_dv[BS + 1];
    __shared__ double s_sl[BS + 1];
    const int base = blockIdx.x * BS;
    const int t = threadIdx.x;
    const int i = base + t;
    const int cnt = min(BS, n - base);
    const bool arc = (model == QEW_MODEL_ARCLENGTH);
#ifdef QEW_BOUNDS_CHECK
    unsigned long long *oob = qew_noise_oob(nz);
#endif
    if (t < cnt) s_h[QEW_IDX(t + 1, BS + 2, oob)] = h[i];
    if (t == 0) s_h[0] = h[base == 0 ? n - 1 : base - 1];
    if (t == cnt - 1) s_h[QEW_IDX(cnt + 1, BS + 2, oob)] = h[(i + 1 == n) ? 0 : i + 1];
    __syncthreads();
    if (t < cnt)
        edge_gradient(nz, i, n, s_h[t + 1], s_h[QEW_IDX(t + 2, BS + 2, oob)], dx, arc,
                      s_dv[QEW_IDX(t + 1, BS + 1, oob)], s_sl[t + 1]);
    if (t == 0) edge_gradient(nz, base == 0 ? n - 1 : base - 1, n, s_h[0], s_h[1], dx, arc, s_dv[0], s_sl[0]);
    __syncthreads();
    if (t < cnt)
        grad[i] = site_gradient(s_h[t], s_h[t + 1], s_h[QEW_IDX(t + 2, BS + 2, oob)], s_dv[t],
                                s_dv[QEW_IDX(t + 1, BS + 1, oob)], s_sl[t], s_sl[t + 1], dx, lt,
                                f, arc);
}

// Objective with a deterministic two-level reduction: fixed grid-stride
// partial sums, CTA tree, per-block partial, and a final tree sum by the last
// block to arrive (ticket counter, reset by that block for the next call).
template <class Noise, class At, int BS>
__global__ void __launch_bounds__(BS)
k_objective(int n, LineDx dx, double lt, double f, int model, Noise nz, At at,
            double *partials, unsigned int *counter, double *out) {
    __shared__ double s_w[BS / 32];
    __shared__ bool s_last;
    double acc = 0.0;
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        acc += edge_energy(nz, i, ip, at(i), at(ip), dx, lt, f, model);
    }
    const double bsum = block_sum<BS>(acc, s_w);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bsum;
        __threadfence();
        const unsigned int ticket = atomicAdd(counter, 1u);
        s_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        double v = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += BS) v += __ldcg(partials + b);
        const double tot = block_sum<BS>(v, s_w);
        if (threadIdx.x == 0) {
            *out = tot;
            *counter = 0u;
        }
    }
}

// Model-layer entry points used by the solvers (qew_model.cu).
qew_status qew_gradient_enqueue(qew_ctx *ctx, const qew_field *field, const double *d_h, int n,
                                const qew_params *p, int precision, double *d_grad);
// FP32 split-index gather with FP64 heights in and FP64 gradient out.
qew_status qew_gradient_split_enqueue(qew_ctx *ctx, const qew_field *field, const double *d_h,
                                      int n, const qew_params *p, double *d_grad);
