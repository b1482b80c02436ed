// qew_split.cu -- FP32 split-index gather: the bandwidth form of gradient().
//
// Same algorithm as the FP64 gradient (qew_model.h:149-193, fused into one
// kernel), with
//   * an FP32 copy of the x-fastest B-spline coefficients (4 B per tap),
//   * heights carried as an integer cell index plus an FP32 fraction in field
//     y-cells, h = (cell + frac) * dy, so no FP64 arithmetic is needed: the
//     edge midpoint (h_i + h_ip)/2 and the elastic differences are formed from
//     exact integer cell sums plus FP32 fraction sums,
//   * edge x positions from integer arithmetic when the line and the field
//     share their resolution and length (gx = e + 1/2 exactly), FP64 only in
//     the general case,
//   * on such a shared grid, when the field holds the x-filtered store
//     (QEW_STORE_FP32_EDGE), the x half of the stencil sum read as one
//     precomputed value per row: 4 taps per edge instead of 16, the same
//     rows and so the same DRAM bytes, a quarter of the load instructions.
// Error against the FP64 form is FP32 rounding of the field, weights and sums
// (about 1e-6 of the gradient's scale; the tests state the bound).
#include <algorithm>
#include <climits>
#include <cmath>

#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"
#include "qew_split.cuh"
#include "qew_tune.cuh"

namespace {

constexpr int kBS = 256;

__device__ __forceinline__ void bsw_value_f(float t, float w[4]) {
    const float s6 = 1.0f / 6.0f;
    const float t2 = t * t, t3 = t2 * t, omt = 1.0f - t;
    w[0] = omt * omt * omt * s6;
    w[1] = (4.0f - 6.0f * t2 + 3.0f * t3) * s6;
    w[2] = (1.0f + 3.0f * t + 3.0f * t2 - 3.0f * t3) * s6;
    w[3] = t3 * s6;
}
__device__ __forceinline__ void bsw_deriv_f(float t, float dw[4]) {
    const float t2 = t * t, omt = 1.0f - t;
    dw[0] = -0.5f * omt * omt;
    dw[1] = -2.0f * t + 1.5f * t2;
    dw[2] = 0.5f + t - 1.5f * t2;
    dw[3] = 0.5f * t2;
}

__device__ __forceinline__ int wrap_cell(int c, int n) {
    if ((unsigned)c >= (unsigned)n) {
        c %= n;
        if (c < 0) c += n;
    }
    return c;
}

// x cell and fraction of the midpoint of edge (e, e+1 mod n).
__device__ __forceinline__ void edge_x(const SplitGeom &g, int e, int &ix, float &fx) {
    if (g.same_grid) {  // n == nx and P == Lx: gx = e + 1/2, wrap edge (n-1)/2
        if (e + 1 < g.n) {
            ix = e;
            fx = 0.5f;
        } else {
            ix = (g.n - 1) >> 1;
            fx = ((g.n - 1) & 1) ? 0.5f : 0.0f;
        }
        return;
    }
    const int ep = (e + 1 == g.n) ? 0 : e + 1;
    double gx = (double)(e + ep) * g.half_ratio;
    const double nd = (double)g.nx;
    if (!(gx >= 0.0 && gx < nd)) gx -= floor(gx / nd) * nd;
    int c = (int)floor(gx);
    if (c >= g.nx) {
        c -= g.nx;
        gx -= nd;
    }
    fx = (float)(gx - (double)c);
    ix = min(max(c, 0), g.nx - 1);
}

// dV/dy at (ix + fx, cy + fy) cells on FP32 coefficients (any stencil,
// wrapping around the field on either axis).
__device__ __forceinline__
float split_dvdy(const float *__restrict__ coef, int nx, int ny, int ix, float fx, int cy,
                 float fy, float inv_dy QEW_OOB_PARAMS) {
    int xs[4], ys[4];
    wrap4(ix, nx, xs);
    wrap4(wrap_cell(cy, ny), ny, ys);
    float wx[4], dwy[4];
    bsw_value_f(fx, wx);
    bsw_deriv_f(fy, dwy);
    float dg = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const float *row = coef + (size_t)ys[b] * (size_t)nx;
        const float r = wx[0] * QEW_LDGP(row + xs[0], coef, oob_n, oob) +
                        wx[1] * QEW_LDGP(row + xs[1], coef, oob_n, oob) +
                        wx[2] * QEW_LDGP(row + xs[2], coef, oob_n, oob) +
                        wx[3] * QEW_LDGP(row + xs[3], coef, oob_n, oob);
        dg += dwy[b] * r;
    }
    return dg * inv_dy;
}

// The same sum for a stencil that wraps neither axis (1 <= ix <= nx - 3,
// 1 <= cy <= ny - 3, true for all but the edge cells): one base pointer, the
// 16 taps at fixed offsets from it, no wrap arithmetic. Same operations in the
// same order as split_dvdy, so the result is identical.
__device__ __forceinline__ float split_dvdy_interior(const float *__restrict__ coef, int nx,
                                                     int ix, const float wx[4], int cy, float fy,
                                                     float inv_dy QEW_OOB_PARAMS) {
    float dwy[4];
    bsw_deriv_f(fy, dwy);
    const float *p = coef + ((size_t)(cy - 1) * (size_t)nx + (size_t)(ix - 1));
    float dg = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const float *row = p + (size_t)b * (size_t)nx;
        const float r = wx[0] * QEW_LDGP(row, coef, oob_n, oob) +
                        wx[1] * QEW_LDGP(row + 1, coef, oob_n, oob) +
                        wx[2] * QEW_LDGP(row + 2, coef, oob_n, oob) +
                        wx[3] * QEW_LDGP(row + 3, coef, oob_n, oob);
        dg += dwy[b] * r;
    }
    return dg * inv_dy;
}

// dV/dy at the midpoint of edge e on a shared grid from the x-filtered store
// E (E[j][e] = sum_a w_a(1/2) c[j][e - 1 + a]): the remaining sum over the 4
// stencil rows, one tap each. The interior form (1 <= cy <= ny - 3) indexes
// from one base pointer; the other wraps the rows.
__device__ __forceinline__ float split_dvdy_edge_interior(const float *__restrict__ E, int nx,
                                                          int e, int cy, float fy,
                                                          float inv_dy QEW_OOB_PARAMS) {
    float dwy[4];
    bsw_deriv_f(fy, dwy);
    const float *p = E + ((size_t)(cy - 1) * (size_t)nx + (size_t)e);
    float dg = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b) dg += dwy[b] * QEW_LDGP(p + (size_t)b * (size_t)nx, E, oob_n, oob);
    return dg * inv_dy;
}
__device__ __forceinline__ float split_dvdy_edge(const float *__restrict__ E, int nx, int ny,
                                                 int e, int cy, float fy,
                                                 float inv_dy QEW_OOB_PARAMS) {
    int ys[4];
    wrap4(wrap_cell(cy, ny), ny, ys);
    float dwy[4];
    bsw_deriv_f(fy, dwy);
    float dg = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b)
        dg += dwy[b] * QEW_LDGP(E + (size_t)ys[b] * (size_t)nx + (size_t)e, E, oob_n, oob);
    return dg * inv_dy;
}

// Midpoint of two split heights: (c0 + f0 + c1 + f1) / 2 as (cell, frac).
__device__ __forceinline__ void split_mid(int c0, float f0, int c1, float f1, int &cm, float &fm) {
    const int C = c0 + c1;
    float F = f0 + f1;       // [0, 2)
    cm = C >> 1;             // floor(C / 2)
    if (C & 1) F += 1.0f;    // odd sum: carry half a cell
    fm = 0.5f * F;           // [0, 1.5)
    if (fm >= 1.0f) {
        fm -= 1.0f;
        cm += 1;
    }
}

// Edge e of a tile, between height slots `slot` and `slot + 1`: writes dV/dy
// at the edge midpoint to dv[slot] and, for the arclength model, the slope
// term s / sqrt(1 + s^2) to sl[slot]. kStore: the caller guarantees g.edge
// (the x-filtered store applies), so only the wrap edge takes the general path.
template <bool kStore>
__device__ __forceinline__ void split_edge(const SplitGeom &g, const float wx_half[4], int e,
                                           const int *sc, const float *sf, int slot, float *dv,
                                           float *sl) {
    int cm;
    float fm;
#ifdef QEW_BOUNDS_CHECK
    const size_t oob_n = (size_t)g.nx * (size_t)g.ny;
#endif
    split_mid(sc[slot], sf[slot], sc[slot + 1], sf[slot + 1], cm, fm);
    const bool y_inner = (cm >= 1 && cm <= g.ny - 3);
    if ((kStore || g.edge) && e + 1 < g.n) {  // x-filtered store: 4 taps (the wrap edge sits at (n-1)/2)
        dv[slot] = y_inner ? split_dvdy_edge_interior(g.edge, g.nx, e, cm, fm, g.inv_dy_f
                                                      QEW_OOB_ARGS(oob_n, g.oob))
                           : split_dvdy_edge(g.edge, g.nx, g.ny, e, cm, fm, g.inv_dy_f
                                             QEW_OOB_ARGS(oob_n, g.oob));
    } else {
        int ix;
        float fx;
        edge_x(g, e, ix, fx);
        if (y_inner && ix >= 1 && ix <= g.nx - 3) {
            float wx[4];
            if (g.same_grid && e + 1 < g.n) {
#pragma unroll
                for (int a = 0; a < 4; ++a) wx[a] = wx_half[a];
            } else {
                bsw_value_f(fx, wx);
            }
            dv[slot] = split_dvdy_interior(g.coef, g.nx, ix, wx, cm, fm, g.inv_dy_f
                                           QEW_OOB_ARGS(oob_n, g.oob));
        } else {
            dv[slot] = split_dvdy(g.coef, g.nx, g.ny, ix, fx, cm, fm, g.inv_dy_f
                                  QEW_OOB_ARGS(oob_n, g.oob));
        }
    }
    if (g.arc) {
        const float dh = ((float)(sc[slot + 1] - sc[slot]) + (sf[slot + 1] - sf[slot])) * g.dy_over_dx;
        sl[slot] = dh * rsqrtf(1.0f + dh * dh);
    }
}

// Gradient at tile site j (height slot j + 1) from the heights either side
// and the two edges that meet there (qew_model.h:177-193).
__device__ __forceinline__ float split_site(const SplitGeom &g, const int *sc, const float *sf,
                                            const float *dv, const float *sl, int j) {
    float line_force;
    if (!g.arc) {
        const float d2 = (float)(sc[j] + sc[j + 2] - 2 * sc[j + 1]) +
                         (sf[j] + sf[j + 2] - 2.0f * sf[j + 1]);
        line_force = -g.lt_dy_over_dx2 * d2;
    } else {
        line_force = g.lt_over_dx * (sl[j] - sl[j + 1]);
    }
    return g.dx_f * (line_force + 0.5f * (dv[j] + dv[j + 1]) - g.f);
}

// One CTA covers a tile of kTile = kBS * kItems consecutive sites of one line
// (blockIdx.y selects the line of a batch stored contiguously, n apart).
// Thread t owns sites t, t + kBS, ... of the tile, so every load phase is
// coalesced, and each thread keeps kItems x 16 independent gathers in flight.
// Sites per thread and the resident-CTA hint are build-time tuning knobs
// (chosen by measurement on GB300; see the build's flags).
#ifndef QEW_SPLIT_ITEMS
#define QEW_SPLIT_ITEMS 2
#endif
#ifndef QEW_SPLIT_MIN_CTAS
#define QEW_SPLIT_MIN_CTAS 8
#endif
constexpr int kItems = QEW_SPLIT_ITEMS;
constexpr int kTile = kBS * kItems;

template <bool IN64, bool OUT64>
__global__ void __launch_bounds__(kBS, QEW_SPLIT_MIN_CTAS)
k_gradient_split(const double *__restrict__ h64, const int *__restrict__ hc,
                 const float *__restrict__ hf, SplitGeom g, double *__restrict__ grad64,
                 float *__restrict__ grad32) {
    __shared__ int s_c[kTile + 2];
    __shared__ float s_f[kTile + 2];
    __shared__ float s_dv[kTile + 1];
    __shared__ float s_sl[kTile + 1];
    const int n = g.n;
    const size_t line = (size_t)blockIdx.y * (size_t)n;
    if (IN64) h64 += line; else { hc += line; hf += line; }
    if (OUT64) grad64 += line; else grad32 += line;
    const int base = blockIdx.x * kTile;
    const int t = threadIdx.x;
    const int cnt = min(kTile, n - base);
    auto load = [&](int site, int slot) {
        if (IN64) {
            const double y = __ldcs(h64 + site);
            const double gy = g.dy_pow2 ? y * g.inv_dy : y / g.dy;
            const double fl = floor(gy);
            s_c[slot] = (int)fl;
            s_f[slot] = (float)(gy - fl);
        } else {
            s_c[slot] = __ldcs(hc + site);
            s_f[slot] = __ldcs(hf + site);
        }
    };
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int j = t + k * kBS;
        if (j < cnt) load(base + j, j + 1);
    }
    if (t == 0) load(base == 0 ? n - 1 : base - 1, 0);
    if (t == kBS - 1) load((base + cnt == n) ? 0 : base + cnt, cnt + 1);
    __syncthreads();
    float wx_half[4];  // x weights at fx = 1/2, every edge but the wrap edge on a shared grid
    bsw_value_f(0.5f, wx_half);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int j = t + k * kBS;
        if (j < cnt) split_edge<false>(g, wx_half, base + j, s_c, s_f, j + 1, s_dv, s_sl);
    }
    if (t == kBS - 1)
        split_edge<false>(g, wx_half, base == 0 ? n - 1 : base - 1, s_c, s_f, 0, s_dv, s_sl);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const int j = t + k * kBS;
        if (j >= cnt) break;
        const float gr = split_site(g, s_c, s_f, s_dv, s_sl, j);
        if (OUT64)
            __stcs(grad64 + base + j, (double)gr);
        else
            __stcs(grad32 + base + j, gr);
    }
}

// 4-byte asynchronous global -> shared copy (completes in the background;
// cp.async.wait_all waits for the calling thread's own copies).
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}

// Persistent form of the split-heights -> FP32 launch: each CTA walks tiles
// gridDim.x apart; the next tile's heights are copied asynchronously into the
// spare shared buffer while the current tile's gathers are in flight, so the
// height round trip leaves the critical path. Same arithmetic as
// k_gradient_split, so the same results bit for bit. Used with the x-filtered
// store, where it measured faster (60.7 vs 63.8 us for 8 lines of 2^20
// points); with the 16-tap gather it measured slower (86.2 vs 81.4 us).
template <int kItems>
__global__ void __launch_bounds__(kBS, QEW_SPLIT_MIN_CTAS)
k_gradient_split_persist(const int *__restrict__ hc, const float *__restrict__ hf, SplitGeom g,
                      float *__restrict__ grad, int count) {
    constexpr int kTile = kBS * kItems;
    __shared__ int s_c[2][kTile + 2];
    __shared__ float s_f[2][kTile + 2];
    __shared__ float s_dv[kTile + 1];
    __shared__ float s_sl[kTile + 1];
    const int n = g.n;
    const int per_line = (n + kTile - 1) / kTile;
    const int t = threadIdx.x;
    // This CTA's tiles are blockIdx.x + k * gridDim.x in line-major order;
    // their (line, index in line) advance by a fixed step, one division per CTA.
    const int step_l = (int)gridDim.x / per_line;
    const int step_i = (int)gridDim.x - step_l * per_line;
    auto fetch = [&](int line, int idx, int buf) {  // heights of a tile (+ halo) into buffer buf
        const int base = idx * kTile;
        const int cnt = min(kTile, n - base);
        const int *c = hc + (size_t)line * (size_t)n;
        const float *f = hf + (size_t)line * (size_t)n;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = t + k * kBS;
            if (j < cnt) {
                cp_async4(&s_c[buf][j + 1], c + base + j);
                cp_async4(&s_f[buf][j + 1], f + base + j);
            }
        }
        if (t == 0) {
            const int site = base == 0 ? n - 1 : base - 1;
            cp_async4(&s_c[buf][0], c + site);
            cp_async4(&s_f[buf][0], f + site);
        } else if (t == kBS - 1) {
            const int site = (base + cnt == n) ? 0 : base + cnt;
            cp_async4(&s_c[buf][cnt + 1], c + site);
            cp_async4(&s_f[buf][cnt + 1], f + site);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    float wx_half[4];
    bsw_value_f(0.5f, wx_half);
    int line = (int)blockIdx.x / per_line;
    int idx = (int)blockIdx.x - line * per_line;
    if (line < count) fetch(line, idx, 0);
    for (int buf = 0; line < count; buf ^= 1) {
        int nline = line + step_l, nidx = idx + step_i;
        if (nidx >= per_line) {
            nidx -= per_line;
            ++nline;
        }
        const int base = idx * kTile;
        const int cnt = min(kTile, n - base);
        const int *sc = s_c[buf];
        const float *sf = s_f[buf];
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        // Barrier A: this tile's heights (every thread's copies) are in place,
        // and every thread has left the previous tile, whose buffer (the
        // other one) may now be refilled and whose edges may be rewritten.
        __syncthreads();
        if (nline < count) fetch(nline, nidx, buf ^ 1);
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = t + k * kBS;
            if (j < cnt) split_edge<true>(g, wx_half, base + j, sc, sf, j + 1, s_dv, s_sl);
        }
        if (t == kBS - 1)
            split_edge<true>(g, wx_half, base == 0 ? n - 1 : base - 1, sc, sf, 0, s_dv, s_sl);
        __syncthreads();  // barrier B: edges done
        float *out = grad + (size_t)line * (size_t)n + base;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = t + k * kBS;
            if (j >= cnt) break;
            __stcs(out + j, split_site(g, sc, sf, s_dv, s_sl, j));
        }
        line = nline;
        idx = nidx;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

__global__ void k_split_heights(const double *__restrict__ h, int n, double dy, double inv_dy,
                                int dy_pow2, int *__restrict__ cell, float *__restrict__ frac) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double gy = dy_pow2 ? h[i] * inv_dy : h[i] / dy;
    const double fl = floor(gy);
    cell[i] = (int)fl;
    frac[i] = (float)(gy - fl);
}

__global__ void k_join_heights(const int *__restrict__ cell, const float *__restrict__ frac, int n,
                               double dy, double *__restrict__ h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) h[i] = ((double)cell[i] + (double)frac[i]) * dy;
}

}  // namespace

SplitGeom qew_split_geom(const qew_field *f, int n, const qew_params *p) {
    SplitGeom g{};
    g.coef = f->coef32;
    g.n = n;
    g.nx = f->nx;
    g.ny = f->ny;
    g.same_grid = (n == f->nx && p->physical_size == f->Lx) ? 1 : 0;
    g.edge = g.same_grid ? f->edge32 : nullptr;
    g.half_ratio = 0.5 * (p->physical_size / n) / f->dx;
    g.dy = f->dy;
    g.inv_dy = 1.0 / f->dy;
    g.dy_pow2 = qew_is_pow2(f->dy) ? 1 : 0;
    const double dx = p->physical_size / n;
    g.inv_dy_f = (float)(1.0 / f->dy);
    g.dy_over_dx = (float)(f->dy / dx);
    g.lt_dy_over_dx2 = (float)(p->line_tension * f->dy / (dx * dx));
    g.lt_over_dx = (float)(p->line_tension / dx);
    g.dx_f = (float)dx;
    g.f = (float)p->driving_force;
    g.arc = (p->model == QEW_MODEL_ARCLENGTH) ? 1 : 0;
#ifdef QEW_BOUNDS_CHECK
    g.oob = qew_bounds_words();
#endif
    return g;
}

// Split heights in, FP32 gradient out, `count` lines n apart.
static qew_status split_launch(qew_ctx *ctx, const SplitGeom &g, int count, const int32_t *d_cell,
                               const float *d_frac, float *d_grad, const char *what) {
    if (g.edge) {  // persistent CTAs, the launch shape chosen by the autotuner
        // Candidates: sites per thread {1, 2} x resident CTAs per SM {4, 6, 8};
        // the per-site arithmetic does not depend on them, so every candidate
        // gives the same bits. Hand-chosen default: 2 sites x 8 CTAs.
        static const char *const names[6] = {"1 site x 4 CTA/SM", "1 site x 6 CTA/SM",
                                              "1 site x 8 CTA/SM", "2 sites x 4 CTA/SM",
                                              "2 sites x 6 CTA/SM", "2 sites x 8 CTA/SM"};
        auto launch = [&](int c) -> qew_status {
            const int items = 1 + c / 3;
            const int ctas = 4 + 2 * (c % 3);
            const long long tiles =
                (long long)((g.n + kBS * items - 1) / (kBS * items)) * count;
            if (tiles > INT_MAX)
                return qew_fail(ctx, QEW_ERR_INVALID, "%s: more than 2^31 tiles", what);
            const int grid = (int)std::min<long long>(tiles, (long long)ctas * ctx->num_sms);
            if (items == 1)
                k_gradient_split_persist<1><<<grid, kBS, 0, ctx->stream>>>(d_cell, d_frac, g,
                                                                           d_grad, count);
            else
                k_gradient_split_persist<2><<<grid, kBS, 0, ctx->stream>>>(d_cell, d_frac, g,
                                                                           d_grad, count);
            return qew_launch_check(ctx, what);
        };
        int cand = 5;
        QEW_TRY(qew_tune_pick(ctx, kTuneGradientSplit,
                              qew_tune_class((long long)g.n * count, g.arc), 6, 5, names, launch,
                              &cand));
        return launch(cand);
    } else {
        k_gradient_split<false, false>
            <<<dim3((g.n + kTile - 1) / kTile, count), kBS, 0, ctx->stream>>>(
                nullptr, d_cell, d_frac, g, nullptr, d_grad);
    }
    return qew_launch_check(ctx, what);
}

static qew_status split_check(qew_ctx *ctx, const qew_field *f, int n, const qew_params *p) {
    if (!ctx || !f || !p || n < 1)
        return qew_fail(ctx, QEW_ERR_INVALID, "split gradient: bad arguments");
    if (f->kind != QEW_FIELD_BSPLINE || !f->coef32)
        return qew_fail(ctx, QEW_ERR_INVALID,
                        "split gradient: needs a B-spline field stored with QEW_STORE_FP32");
    return QEW_OK;
}

qew_status qew_gradient_split_enqueue(qew_ctx *ctx, const qew_field *f, const double *d_h, int n,
                                      const qew_params *p, double *d_grad) {
    QEW_TRY(split_check(ctx, f, n, p));
    const SplitGeom g = qew_split_geom(f, n, p);
    k_gradient_split<true, true><<<dim3((n + kTile - 1) / kTile, 1), kBS, 0, ctx->stream>>>(
        d_h, nullptr, nullptr, g, d_grad, nullptr);
    return qew_launch_check(ctx, "gradient_split64");
}

extern "C" {

qew_status qew_split_heights(qew_ctx *ctx, const qew_field *f, const double *d_h, int n,
                             int32_t *d_cell, float *d_frac) {
    QEW_RANGE();
    if (!ctx || !f || !d_h || !d_cell || !d_frac || n < 1 || f->kind != QEW_FIELD_BSPLINE)
        return qew_fail(ctx, QEW_ERR_INVALID, "split_heights: bad arguments");
    k_split_heights<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
        d_h, n, f->dy, 1.0 / f->dy, qew_is_pow2(f->dy) ? 1 : 0, d_cell, d_frac);
    return qew_launch_check(ctx, "split_heights");
}

qew_status qew_join_heights(qew_ctx *ctx, const qew_field *f, const int32_t *d_cell,
                            const float *d_frac, int n, double *d_h) {
    QEW_RANGE();
    if (!ctx || !f || !d_h || !d_cell || !d_frac || n < 1 || f->kind != QEW_FIELD_BSPLINE)
        return qew_fail(ctx, QEW_ERR_INVALID, "join_heights: bad arguments");
    k_join_heights<<<(n + 255) / 256, 256, 0, ctx->stream>>>(d_cell, d_frac, n, f->dy, d_h);
    return qew_launch_check(ctx, "join_heights");
}

qew_status qew_gradient_split(qew_ctx *ctx, const qew_field *f, const int32_t *d_cell,
                              const float *d_frac, int n, const qew_params *p, float *d_grad) {
    QEW_RANGE();
    QEW_TRY(split_check(ctx, f, n, p));
    if (!d_cell || !d_frac || !d_grad)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient_split: null buffer");
    return split_launch(ctx, qew_split_geom(f, n, p), 1, d_cell, d_frac, d_grad, "gradient_split");
}

qew_status qew_gradient_split_batch(qew_ctx *ctx, const qew_field *f, int count,
                                    const int32_t *d_cell, const float *d_frac, int n,
                                    const qew_params *p, float *d_grad) {
    QEW_RANGE();
    QEW_TRY(split_check(ctx, f, n, p));
    if (!d_cell || !d_frac || !d_grad || count < 1 || count > 65535)
        return qew_fail(ctx, QEW_ERR_INVALID, "gradient_split_batch: bad arguments");
    return split_launch(ctx, qew_split_geom(f, n, p), count, d_cell, d_frac, d_grad,
                        "gradient_split_batch");
}

}  // extern "C"
