// qew_poly.cu -- FP64 gradient on the cell-polynomial store (QEW_STORE_FP64_POLY).
//
// gradient() (qew_model.h:149-193) of lines with one point per field column,
// in FP64 throughout: the edge pass reads one 32-byte cell of the store per
// edge (the x-filtered field's cubic in the row fraction, built once with the
// field) and evaluates dV/dy with two FMAs; the per-site combine is the
// reference's, with its factors folded:
//   grad_i = dx (F_el,i + (dv_{i-1} + dv_i)/2 - f)
//          = c_el d2h_i + (dx/2)(dv_{i-1} + dv_i) - dx f        (linear,
//            c_el = -Gamma/dx, d2h_i = (h_{i-1} + h_{i+1}) - 2 h_i as the reference forms it)
//          = Gamma (s_{i-1} - s_i) + (dx/2)(dv_{i-1} + dv_i) - dx f  (arclength).
// The row cell and fraction of each edge midpoint come from the bits of
// h_e + h_{e+1} when the row spacing is a power of two (qew_poly.cuh), so an
// edge of the linear model costs 3 FP64 instructions and a site 5.
//
// At f = 0 with dx/2 a power of two 2^k (kF0) the combine's first term is an
// exact scaling: (dx/2)(dv_{i-1} + dv_i) == dv'_{i-1} + dv'_i bit for bit
// with dv' = 2^k dv, and each edge forms dv' by adding k to the exponent
// field of dv (integer instructions; the FP64 multiply where dv or dv' is
// zero, subnormal or non-finite). A site then costs 4 FP64 instructions
// instead of 5.
//
// Launch: persistent, batched (lines stored n apart), one CTA per resident
// slot; each CTA walks tiles of kTile sites gridDim.x apart and copies the
// next tile's heights into its spare shared buffer with cp.async while the
// current tile's gathers are in flight. The wrap edge of each line (at
// x = (n - 1) dx / 2, not a half-integer column) takes the 16-tap path.
#include <algorithm>
#include <climits>
#include <cmath>

#include "qew_internal.cuh"
#include "qew_poly.cuh"
#include "qew_tune.cuh"

namespace {

constexpr int kBS = 256;
constexpr int kMinCtas = 4;  // 64 registers a thread: up to 4 resident CTAs per SM

struct PolyGeom {
    const double *poly;   // [ny][nx][4]
    NoiseBSpline64 nz;    // 16-tap path of the wrap edge and the reference's fold
    int n;
    int ky;               // (h_e + h_ep) * 2^ky = midpoint in row cells, or kPolyNotPow2
    double half_inv_dy;   // 0.5 / dy when the spacing is not a power of two
    LineDx L;
    double c_el;          // -Gamma / dx
    double lt;            // Gamma
    double half_dx, fdx;  // dx / 2, dx f
    int half_dx_exp;      // k with dx / 2 == 2^k (the kF0 form)
};

// v * scale for a zero, subnormal or non-finite v or result: a call of its
// own, so the compiler cannot evaluate the multiply for every lane and
// select (which would put the FP64 instruction back on every edge).
__device__ __noinline__ double scale_pow2_slow(double v, double scale) { return v * scale; }

// v * 2^k (scale == 2^k), exact: the exponent field moves by k when v and
// the result are normal.
__device__ __forceinline__ double scale_pow2(double v, int k, double scale) {
    const int hi = __double2hiint(v);
    const int e = (hi >> 20) & 0x7FF;
    if (e != 0 && e + k >= 1 && e + k <= 2046)
        return __hiloint2double(hi + (k << 20), __double2loint(v));
    return scale_pow2_slow(v, scale);
}

// dV/dy at the midpoint of edge (e, e + 1 mod n) of heights he, hep.
__device__ __forceinline__ double poly_edge_dvdy(const PolyGeom &g, int e, double he,
                                                 double hep) {
    const double a = hep + he;  // the reference's (h_ip + h_i), qew_model.h:168
    if (e + 1 < g.n) {
        int iy;
        double t;
        poly_locate(a, g.ky, g.half_inv_dy, g.nz, iy, t);
        iy = QEW_IDX(iy, g.nz.ny, g.nz.oob);
        e = QEW_IDX(e, g.nz.nx, g.nz.oob);
        double q0, q1, q2;
        poly_load3(g.poly + ((size_t)iy * (size_t)g.nz.nx + (size_t)e) * 4, q0, q1, q2);
        return poly_dvdy(q0, q1, q2, t);
    }
    const double xc = (double)e * 0.5 * g.L.dx;  // (i + ip) dx / 2 with ip = 0
    return g.nz.dvdy(xc, a * 0.5);
}

// 8-byte asynchronous global -> shared copy.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

template <bool kArc, int kItems, bool kF0>
__global__ void __launch_bounds__(kBS, kMinCtas)
k_gradient_poly(const double *__restrict__ h, PolyGeom g, double *__restrict__ grad, int count) {
    constexpr int kTile = kBS * kItems;
    __shared__ double s_h[2][kTile + 2];
    __shared__ double s_dv[kTile + 1];
    __shared__ double s_sl[kArc ? kTile + 1 : 1];
    const int n = g.n;
    const int per_line = (n + kTile - 1) / kTile;
    const int t = threadIdx.x;
    // This CTA's tiles are blockIdx.x + k * gridDim.x in line-major order;
    // (line, index in line) advance by a fixed step, one division per CTA.
    const int step_l = (int)gridDim.x / per_line;
    const int step_i = (int)gridDim.x - step_l * per_line;
    auto fetch = [&](int line, int idx, int buf) {  // a tile's heights (+ halo) into buffer buf
        const int base = idx * kTile;
        const int cnt = min(kTile, n - base);
        const double *hl = h + (size_t)line * (size_t)n;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = t + k * kBS;
            if (j < cnt) cp_async8(&s_h[buf][j + 1], hl + base + j);
        }
        if (t == 0) {
            cp_async8(&s_h[buf][0], hl + (base == 0 ? n - 1 : base - 1));
        } else if (t == kBS - 1) {
            cp_async8(&s_h[buf][cnt + 1], hl + ((base + cnt == n) ? 0 : base + cnt));
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
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
        const double *sh = s_h[buf];
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        // Barrier A: this tile's heights are in place, and every thread has
        // left the previous tile, whose buffer may now be refilled and whose
        // edge values may be rewritten.
        __syncthreads();
        if (nline < count) fetch(nline, nidx, buf ^ 1);
        auto edge = [&](int e, int slot) {
            slot = QEW_IDX(slot, kTile + 1, g.nz.oob);
            const double he = sh[slot], hep = sh[slot + 1];
            const double dv = poly_edge_dvdy(g, e, he, hep);
            s_dv[slot] = kF0 ? scale_pow2(dv, g.half_dx_exp, g.half_dx) : dv;
            if (kArc) {
                const double dh = g.L.div(hep - he);
                s_sl[slot] = dh * rsqrt(1.0 + dh * dh);
            }
        };
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = t + k * kBS;
            if (j < cnt) edge(base + j, j + 1);
        }
        if (t == kBS - 1) edge(base == 0 ? n - 1 : base - 1, 0);
        __syncthreads();  // barrier B: edge values in place
        double *out = grad + (size_t)line * (size_t)n + base;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const int j = QEW_IDX(t + k * kBS, kTile, g.nz.oob);
            if (t + k * kBS >= cnt) break;
            const double rest = kF0 ? s_dv[j] + s_dv[j + 1]
                                    : fma(g.half_dx, s_dv[j] + s_dv[j + 1], -g.fdx);
            double gr;
            if (kArc) {
                gr = fma(g.lt, s_sl[j] - s_sl[j + 1], rest);
            } else {
                const double d2h = fma(-2.0, sh[j + 1], sh[j] + sh[j + 2]);
                gr = fma(g.c_el, d2h, rest);
            }
            __stcs(out + j, gr);
        }
        line = nline;
        idx = nidx;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// {q0, q1, q2, v0} of every (row cell j, column e) from the FP64
// coefficients c ([ny][nx]); see qew_poly.cuh for the formulas. Each thread
// walks kStoreRows row cells of one column and filters each coefficient row
// along x once: cell j takes the filtered values of rows j-1..j+2 from a
// window of four, so a cell costs one x-filter (4 FP64 instructions) and the
// combination (11) instead of four x-filters. FP64-instruction bound.
constexpr int kStoreRows = 32;
constexpr int kStoreBS = 256;

__device__ __forceinline__ double x_filter(const double *__restrict__ r, int em, int e, int ep,
                                           int ep2) {
    const double w0 = 1.0 / 48.0, w1 = 23.0 / 48.0;
    return __fma_rn(w0, __ldg(r + ep2),
                    __fma_rn(w1, __ldg(r + ep), __fma_rn(w1, __ldg(r + e), w0 * __ldg(r + em))));
}

__global__ void __launch_bounds__(kStoreBS) k_poly_store(const double *__restrict__ c, int nx,
                                                         int ny, double inv_dy,
                                                         double *__restrict__ out) {
    const int e = blockIdx.x * kStoreBS + threadIdx.x;
    if (e >= nx) return;
    const int j0 = blockIdx.y * kStoreRows;
    const int j1 = min(ny, j0 + kStoreRows);
    const int em = (e == 0) ? nx - 1 : e - 1;
    const int ep = (e + 1 == nx) ? 0 : e + 1;
    const int ep2 = (ep + 1 == nx) ? 0 : ep + 1;
    const double half_inv_dy = 0.5 * inv_dy, s6 = 1.0 / 6.0;
    int r = (j0 == 0) ? ny - 1 : j0 - 1;  // row j0-1, periodic
    double E0 = x_filter(c + (size_t)r * nx, em, e, ep, ep2);
    r = (r + 1 == ny) ? 0 : r + 1;
    double E1 = x_filter(c + (size_t)r * nx, em, e, ep, ep2);
    r = (r + 1 == ny) ? 0 : r + 1;
    double E2 = x_filter(c + (size_t)r * nx, em, e, ep, ep2);
    for (int j = j0; j < j1; ++j) {
        r = (r + 1 == ny) ? 0 : r + 1;  // row j+2
        const double E3 = x_filter(c + (size_t)r * nx, em, e, ep, ep2);
        const double s02 = E0 + E2;
        const double q0 = (E2 - E0) * half_inv_dy;
        const double q1 = __fma_rn(-2.0, E1, s02) * inv_dy;
        const double q2 = __fma_rn(3.0, E1 - E2, E3 - E0) * half_inv_dy;
        const double v0 = __fma_rn(4.0, E1, s02) * s6;
        double *o = out + ((size_t)j * (size_t)nx + (size_t)e) * 4;  // 32-byte aligned
        asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(o), "d"(q0), "d"(q1),
                     "d"(q2), "d"(v0)
                     : "memory");
        E0 = E1;
        E1 = E2;
        E2 = E3;
    }
}

}  // namespace

bool qew_poly_applies(const qew_field *f, int n, const qew_params *p) {
    return f && f->kind == QEW_FIELD_BSPLINE && f->poly64 && f->coef64 && n == f->nx &&
           p->physical_size == f->Lx;
}

qew_status qew_poly_store_build(qew_ctx *ctx, const double *c, int nx, int ny, double dy,
                                double *out) {
    if ((ny + kStoreRows - 1) / kStoreRows > 65535)
        return qew_fail(ctx, QEW_ERR_INVALID, "poly store: more than 2^21 field rows");
    const dim3 grid((unsigned)((nx + kStoreBS - 1) / kStoreBS),
                    (unsigned)((ny + kStoreRows - 1) / kStoreRows));
    k_poly_store<<<grid, kStoreBS, 0, ctx->stream>>>(c, nx, ny, 1.0 / dy, out);
    return qew_launch_check(ctx, "poly_store");
}

qew_status qew_gradient_poly_enqueue(qew_ctx *ctx, const qew_field *f, int count,
                                     const double *d_h, int n, const qew_params *p,
                                     double *d_grad) {
    if (!qew_poly_applies(f, n, p)) return QEW_ERR_UNSUPPORTED;
    PolyGeom g{};
    g.poly = f->poly64;
    g.nz = make_bspline64(f, n, p->physical_size);
    g.n = n;
    g.ky = poly_scale_exponent(f->dy);
    g.half_inv_dy = 0.5 / f->dy;
    g.L = make_line_dx(p->physical_size, n);
    g.c_el = -p->line_tension / g.L.dx;
    g.lt = p->line_tension;
    g.half_dx = 0.5 * g.L.dx;
    g.fdx = g.L.dx * p->driving_force;
    int hx;
    const bool f0 = p->driving_force == 0.0 && frexp(g.half_dx, &hx) == 0.5;
    g.half_dx_exp = hx - 1;  // half_dx == 2^(hx-1) when f0
    const bool arc = (p->model == QEW_MODEL_ARCLENGTH);
    // Candidates: sites per thread {1, 2, 4} x resident CTAs per SM {2, 3, 4};
    // every one computes the same numbers (the per-site arithmetic does not
    // depend on the tiling). Hand-chosen default: 2 sites, 4 CTAs.
    static const char *const names[9] = {"1 site x 2 CTA/SM", "1 site x 3 CTA/SM",
                                          "1 site x 4 CTA/SM", "2 sites x 2 CTA/SM",
                                          "2 sites x 3 CTA/SM", "2 sites x 4 CTA/SM",
                                          "4 sites x 2 CTA/SM", "4 sites x 3 CTA/SM",
                                          "4 sites x 4 CTA/SM"};
    auto launch = [&](int c) -> qew_status {
        const int items = 1 << (c / 3);
        const int ctas = 2 + c % 3;
        const long long tiles = (long long)((n + kBS * items - 1) / (kBS * items)) * count;
        if (tiles > INT_MAX)
            return qew_fail(ctx, QEW_ERR_INVALID, "gradient: more than 2^31 tiles");
        const int grid = (int)std::min<long long>(tiles, (long long)ctas * ctx->num_sms);
#define QEW_POLY_LAUNCH(A, I, F) \
    k_gradient_poly<A, I, F><<<grid, kBS, 0, ctx->stream>>>(d_h, g, d_grad, count)
#define QEW_POLY_ITEMS(A, F)                       \
    if (items == 1) QEW_POLY_LAUNCH(A, 1, F);      \
    else if (items == 2) QEW_POLY_LAUNCH(A, 2, F); \
    else QEW_POLY_LAUNCH(A, 4, F)
        if (arc) {
            if (f0) { QEW_POLY_ITEMS(true, true); } else { QEW_POLY_ITEMS(true, false); }
        } else {
            if (f0) { QEW_POLY_ITEMS(false, true); } else { QEW_POLY_ITEMS(false, false); }
        }
#undef QEW_POLY_ITEMS
#undef QEW_POLY_LAUNCH
        return qew_launch_check(ctx, "gradient_poly");
    };
    int cand = 5;
    QEW_TRY(qew_tune_pick(ctx, kTuneGradientPoly,
                          qew_tune_class((long long)n * count, (arc ? 1 : 0) + (f0 ? 2 : 0)), 9,
                          5, names, launch,
                          &cand));
    return launch(cand);
}
