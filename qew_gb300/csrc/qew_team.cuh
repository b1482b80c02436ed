// qew_team.cuh -- the group of threads that runs one device-resident solve:
// one CTA (CtaTeam) or one thread-block cluster (ClusterTeam: up to 16 CTAs
// on as many SMs, sharing a line). A team gives every thread its first index
// and stride over the line, broadcast reductions whose result is identical in
// every thread, and a barrier after which writes of any team thread are
// visible. The solver code (gradient, objective, preconditioner, L-BFGS) is
// written once against this interface.
//   * CtaTeam: exactly the CTA primitives of qew_block.cuh (warp butterflies,
//     warp partials added in warp order, __syncthreads).
//   * ClusterTeam: CTA reduction first, then every CTA publishes its partial
//     into a slot of every CTA's shared memory (distributed shared memory),
//     one cluster barrier, and every CTA adds the partials in rank order --
//     deterministic, and the same value in every CTA without a second
//     round. Slots alternate between two buffers, so a publish never lands
//     on a buffer another CTA may still be reading (it passed the barrier
//     that follows that read). Loads of team-shared vectors bypass L1
//     (ld.global.cg): another SM may have written them.
#pragma once

#include <cooperative_groups.h>

#include "qew_block.cuh"

constexpr int kTeamMaxCtas = 16;

template <int BS>
struct CtaTeam {
    static constexpr bool kCluster = false;
    static constexpr int kBS = BS;
    double *s_w;  // >= 96 doubles of shared memory
    __device__ __forceinline__ int tid() const { return threadIdx.x; }
    __device__ __forceinline__ int stride() const { return BS; }
    __device__ __forceinline__ unsigned rank() const { return 0; }
    __device__ __forceinline__ unsigned size() const { return 1; }
    __device__ __forceinline__ double sum(double v) const { return bsum_all<BS>(v, s_w); }
    __device__ __forceinline__ double max(double v) const { return bmax_all<BS>(v, s_w); }
    __device__ __forceinline__ void sum3(double &a, double &b, double &c) const {
        bsum3_all<BS>(a, b, c, s_w);
    }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ double ld(const double *p) const { return *p; }
    __device__ __forceinline__ float ld(const float *p) const { return *p; }
};

template <int BS>
struct ClusterTeam {
    static constexpr bool kCluster = true;
    static constexpr int kBS = BS;
    double *s_w;    // >= 96 doubles of shared memory
    double *s_red;  // 2 x 3 x kTeamMaxCtas doubles of shared memory
    unsigned r, sz;
    int phase = 0;
    __device__ __forceinline__ int tid() const { return (int)r * BS + threadIdx.x; }
    __device__ __forceinline__ int stride() const { return BS * (int)sz; }
    __device__ __forceinline__ unsigned rank() const { return r; }
    __device__ __forceinline__ unsigned size() const { return sz; }
    __device__ __forceinline__ void sync() const { cooperative_groups::this_cluster().sync(); }
    __device__ __forceinline__ double ld(const double *p) const { return __ldcg(p); }
    __device__ __forceinline__ float ld(const float *p) const { return __ldcg(p); }
    // publish k CTA values into every CTA's slots, barrier; returns the local slots
    __device__ __forceinline__ double *publish(const double *v, int k) {
        double *buf = s_red + phase * 3 * kTeamMaxCtas;
        phase ^= 1;
        if (threadIdx.x < sz) {
            double *remote = cooperative_groups::this_cluster().map_shared_rank(buf, threadIdx.x);
            for (int j = 0; j < k; ++j) remote[j * kTeamMaxCtas + r] = v[j];
        }
        sync();
        return buf;
    }
    __device__ __forceinline__ double sum(double v) {
        const double c = bsum_all<BS>(v, s_w);
        const double *buf = publish(&c, 1);
        double t = 0.0;
        for (unsigned k = 0; k < sz; ++k) t += buf[k];
        return t;
    }
    __device__ __forceinline__ double max(double v) {
        const double c = bmax_all<BS>(v, s_w);
        const double *buf = publish(&c, 1);
        double t = 0.0;
        for (unsigned k = 0; k < sz; ++k) t = fmax(t, buf[k]);
        return t;
    }
    __device__ __forceinline__ void sum3(double &a, double &b, double &c) {
        bsum3_all<BS>(a, b, c, s_w);
        const double v[3] = {a, b, c};
        const double *buf = publish(v, 3);
        a = b = c = 0.0;
        for (unsigned k = 0; k < sz; ++k) {
            a += buf[k];
            b += buf[kTeamMaxCtas + k];
            c += buf[2 * kTeamMaxCtas + k];
        }
    }
};

// gradient() of a whole line by a team (qew_model.h:149-193): edge pass into
// ev/es, barrier, site combine into g, barrier.
template <class Noise, class Team, class R>
__device__ void team_gradient(Team &T, const Noise &nz, const double *__restrict__ h, int n,
                              const LineDx &dx, double lt, double f, bool arc, R *ev, R *es,
                              R *g) {
    for (int e = T.tid(); e < n; e += T.stride()) {
        const int ep = (e + 1 == n) ? 0 : e + 1;
        double dv, sl;
        edge_gradient(nz, e, n, T.ld(h + e), T.ld(h + ep), dx, arc, dv, sl);
        ev[e] = (R)dv;
        es[e] = (R)sl;
    }
    T.sync();
    for (int i = T.tid(); i < n; i += T.stride()) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const int im = (i == 0) ? n - 1 : i - 1;
        g[i] = (R)site_gradient(T.ld(h + im), T.ld(h + i), T.ld(h + ip), (double)T.ld(ev + im),
                                (double)T.ld(ev + i), (double)T.ld(es + im), (double)T.ld(es + i),
                                dx, lt, f, arc);
    }
    T.sync();
}

// objective() at x0 + alpha*d by a team.
template <class Noise, class Team, class R>
__device__ double team_objective(Team &T, const Noise &nz, const double *__restrict__ x0,
                                 const R *__restrict__ d, double alpha, int n,
                                 const LineDx &dx, double lt, double f, int model) {
    double acc = 0.0;
    for (int i = T.tid(); i < n; i += T.stride()) {
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const double hi = T.ld(x0 + i) + alpha * (double)T.ld(d + i);
        const double hip = T.ld(x0 + ip) + alpha * (double)T.ld(d + ip);
        acc += edge_energy(nz, i, ip, hi, hip, dx, lt, f, model);
    }
    return T.sum(acc);
}

// The periodic recurrence of block_periodic_recurrence over a cluster: the
// chunks are the cluster's threads in rank order; the CTA scan of the chunk
// maps is followed by a scan over the CTAs' aggregate maps (published through
// distributed shared memory), then the periodic closure and the second chunk
// pass. s_b: BS doubles, s_agg: 2 x kTeamMaxCtas doubles. Ends with a barrier.
template <int BS, class R>
__device__ void cluster_periodic_recurrence(ClusterTeam<BS> &T, const R *in, R *out, int n,
                                            bool rev, const PrecondCoef &pc, double *s_b,
                                            double *s_agg) {
    const int t = threadIdx.x;
    const int G = BS * (int)T.size();
    const int c = (n + G - 1) / G;
    const int gt = T.tid();
    const int start = min(gt * c, n);
    const int end = min(start + c, n);
    const int cta_start = min((int)T.rank() * BS * c, n);
    const double z = pc.z;
    double B = 0.0;
    for (int k = start; k < end; ++k) B = (double)__ldcg(in + (rev ? n - 1 - k : k)) + z * B;
    double A = (end > start) ? exp((double)(end - start) * pc.logz) : 1.0;
    double *s_w = T.s_w;
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
    if (w == 0) {
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
    if (w > 0) {
        B = A * s_w[32 + w - 1] + B;
        A = A * s_w[w - 1];
    }
    s_b[t] = B;  // zero-start value at the end of this chunk, from the CTA's start
    __syncthreads();
    // the CTA's aggregate map (the last thread's inclusive prefix), to every CTA
    if (t < (int)T.size()) {
        double *remote = cooperative_groups::this_cluster().map_shared_rank(s_agg, t);
        remote[T.rank()] = exp((double)(min(cta_start + BS * c, n) - cta_start) * pc.logz);
        remote[kTeamMaxCtas + T.rank()] = s_b[BS - 1];
    }
    T.sync();
    double Bp = 0.0, Bt = 0.0;  // zero-start value before this CTA, at the end
    for (unsigned k = 0; k < T.size(); ++k) {
        if (k == T.rank()) Bp = Bt;
        Bt = s_agg[k] * Bt + s_agg[kTeamMaxCtas + k];
    }
    const double P = Bt * pc.inv_1mzn;  // periodic y_{-1}
    const double cin_cta = (t > 0) ? s_b[t - 1] : 0.0;
    const double cin = cin_cta + exp((double)(start - cta_start) * pc.logz) * Bp;
    double y = cin + exp((double)start * pc.logz) * P;
    for (int k = start; k < end; ++k) {
        const int idx = rev ? n - 1 - k : k;
        y = (double)__ldcg(in + idx) + z * y;
        out[idx] = (R)y;
    }
    T.sync();
}

// d = M^{-1} q (lbfgs.h:173-180) by a team.
template <class Team, class R>
__device__ void team_precond(Team &T, const R *q, R *d, int n, const PrecondCoef &pc, double *s_b,
                             double *s_agg) {
    if constexpr (!Team::kCluster) {
        (void)s_agg;
        block_precond<Team::kBS, R>(q, d, n, pc, s_b, T.s_w);
    } else {
        if (pc.scalar) {
            for (int i = T.tid(); i < n; i += T.stride())
                d[i] = (R)((double)__ldcg(q + i) * pc.inv_sigma);
            T.sync();
            return;
        }
        cluster_periodic_recurrence(T, q, d, n, false, pc, s_b, s_agg);
        cluster_periodic_recurrence(T, (const R *)d, d, n, true, pc, s_b, s_agg);
        for (int i = T.tid(); i < n; i += T.stride()) d[i] = (R)((double)__ldcg(d + i) * pc.gain);
        T.sync();
    }
}
