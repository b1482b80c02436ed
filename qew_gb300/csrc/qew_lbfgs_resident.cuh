// qew_lbfgs_resident.cuh -- one CTA runs one complete lbfgs_minimize
// (lbfgs.h:94-287). Shared by the single-line entry point and the batched
// ensemble kernel.
#pragma once

#include "qew_team.cuh"

constexpr int kLbfgsMaxM = 32;
constexpr int kLbfgsVecs = 7;  // g, g_new, d, q, edge dV/dy, edge slope, trial position

struct LbfgsCfg {
    int m;
    double ftol;
    int max_iter;
    double c1;
    double ls_shrink;
    int max_ls;
    double curvature_eps;
    int precondition;
    int ls_fallback;
};

// Approximate-Wolfe test (W. Hager, H. Zhang, SIAM J. Optim. 16 (2005)),
// tried when the Armijo energy test fails: sigma*phi'(0) <= phi'(a) <=
// (2*delta - 1)*phi'(0) and phi(a) <= phi(0) + eps*|phi(0)|. It decides on
// slopes, which keep their relative accuracy where energy differences drown
// in the rounding of |E| (the regime of a ~1e-8 gradient tolerance).
constexpr double kAwDelta = 0.1;
constexpr double kAwSigma = 0.9;
constexpr double kAwEps = 1e-10;

inline LbfgsCfg lbfgs_cfg_from(const qew_lbfgs_params *lp) {
    LbfgsCfg c;
    c.m = lp->m;
    c.ftol = lp->ftol;
    c.max_iter = lp->max_iter;
    c.c1 = lp->c1;
    c.ls_shrink = lp->ls_shrink;
    c.max_ls = lp->max_ls;
    c.curvature_eps = lp->curvature_eps;
    c.precondition = lp->precondition;
    c.ls_fallback = lp->ls_fallback;
    return c;
}

inline size_t lbfgs_block_smem_bytes(int /*bs*/, int /*m*/) { return 0; }

// History bookkeeping of lbfgs.h:107-114, 262-279: `slots` in chronological
// order, and buffer indices standing in for the reference's View swaps.
struct LbfgsShared {
    double rho[kLbfgsMaxM];
    double la[kLbfgsMaxM];
    int slots[kLbfgsMaxM];
    int sbuf[kLbfgsMaxM];
    int ybuf[kLbfgsMaxM];
    int nslots;
    int stmp;
    int ytmp;
};

// Workspace (npad doubles per vector): g, g_new, d, q, ev, es (vectors of
// Real), the trial position xt (FP64), then 2(m+1) history buffers (m S rows
// + spare, m Y rows + spare; Real). Real = float keeps the vectors and their
// dot products in FP32 (a first phase on FP32 coefficients); positions,
// energies, reductions across threads and every scalar stay FP64.
template <class Noise, class Team, class Real = double>
__device__ qew_lbfgs_result lbfgs_team(Team &T, const Noise &nz, double *__restrict__ h,
                                       const int n, const qew_params P, const LbfgsCfg cfg,
                                       const PrecondCoef pc, double *ws, size_t npad) {
    __shared__ double s_b[Team::kBS];
    __shared__ double s_agg[2 * kTeamMaxCtas];
    __shared__ LbfgsShared sh;
    const int t0 = T.tid(), ts = T.stride();
    const LineDx dx = make_line_dx(P.physical_size, n);
    const double lt = P.line_tension, f = P.driving_force;
    const int model = P.model;
    const bool arc = (model == QEW_MODEL_ARCLENGTH);
    Real *g = (Real *)ws, *gn = (Real *)(ws + npad), *d = (Real *)(ws + 2 * npad);
    Real *q = (Real *)(ws + 3 * npad), *ev = (Real *)(ws + 4 * npad), *es = (Real *)(ws + 5 * npad);
    double *xt = ws + 6 * npad;
    double *bufs = ws + (size_t)kLbfgsVecs * npad;
    auto row = [&](int b) { return (Real *)(bufs + (size_t)b * npad); };
    const int m = cfg.m;
    if (threadIdx.x == 0) {
        sh.nslots = 0;
        for (int k = 0; k < m; ++k) {
            sh.sbuf[k] = k;
            sh.ybuf[k] = m + 1 + k;
        }
        sh.stmp = m;
        sh.ytmp = 2 * m + 1;
    }
    T.sync();

    qew_lbfgs_result res;
    res.iterations = 0;
    res.max_force = 0;
    res.converged = 0;
    res.n_func_evals = 0;
    res.n_curvature_skips = 0;
    res.n_ls_restarts = 0;
    double gamma = 1.0;
    int ls_fail_streak = 0;
    double phi = 0.0;
    bool done = false;

    team_gradient<Noise>(T, nz, h, n, dx, lt, f, arc, ev, es, g);

    for (int it = 0; it < cfg.max_iter; ++it) {
        double lm = 0.0;
        for (int i = t0; i < n; i += ts) lm = fmax(lm, fabs((double)g[i]));
        const double gmax = T.max(lm);
        if (gmax < cfg.ftol) {  // lbfgs.h:155-161
            res.iterations = it;
            res.max_force = gmax;
            res.converged = 1;
            done = true;
            break;
        }
        // two-loop recursion, lbfgs.h:163-191
        for (int i = t0; i < n; i += ts) q[i] = g[i];
        T.sync();
        const int hs = sh.nslots;
        for (int idx = hs - 1; idx >= 0; --idx) {
            const int r = sh.slots[idx];
            const Real *S = row(sh.sbuf[r]);
            const Real *Y = row(sh.ybuf[r]);
            Real acc = 0;
            for (int i = t0; i < n; i += ts) acc += S[i] * q[i];
            const double a = sh.rho[r] * T.sum((double)acc);
            if (threadIdx.x == 0) sh.la[idx] = a;
            const Real na = (Real)(-a);
            for (int i = t0; i < n; i += ts) q[i] += na * Y[i];
            T.sync();
        }
        if (cfg.precondition) {
            team_precond(T, q, d, n, pc, s_b, s_agg);
        } else {
            const double g0 = (hs == 0) ? 1.0 : gamma;
            for (int i = t0; i < n; i += ts) d[i] = (Real)(g0 * q[i]);
            T.sync();
        }
        for (int idx = 0; idx < hs; ++idx) {
            const int r = sh.slots[idx];
            const Real *S = row(sh.sbuf[r]);
            const Real *Y = row(sh.ybuf[r]);
            Real acc = 0;
            for (int i = t0; i < n; i += ts) acc += Y[i] * T.ld(d + i);
            const double b = sh.rho[r] * T.sum((double)acc);
            const Real c = (Real)(sh.la[idx] - b);
            for (int i = t0; i < n; i += ts) d[i] = T.ld(d + i) + c * S[i];
            T.sync();
        }
        // d = -d, fused with dphi0 = g.d (lbfgs.h:190-194)
        Real acc = 0;
        for (int i = t0; i < n; i += ts) {
            const Real v = -T.ld(d + i);
            d[i] = v;
            acc += g[i] * v;
        }
        double dphi0 = T.sum((double)acc);
        bool empty = (hs == 0);
        if (dphi0 >= 0) {  // steepest-descent fallback, lbfgs.h:195-200
            if (threadIdx.x == 0) sh.nslots = 0;
            empty = true;
            Real gg = 0;
            for (int i = t0; i < n; i += ts) {
                d[i] = -g[i];
                gg += g[i] * g[i];
            }
            dphi0 = -T.sum((double)gg);
        }
        // Armijo backtracking, lbfgs.h:202-238
        if (it == 0) {
            phi = team_objective<Noise>(T, nz, h, d, 0.0, n, dx, lt, f, model);
            ++res.n_func_evals;
        }
        const double phi0 = phi;
        double alpha = 1.0;
        if (!cfg.precondition && empty) {
            Real gg = 0;
            for (int i = t0; i < n; i += ts) gg += g[i] * g[i];
            alpha = 1.0 / fmax(1.0, sqrt(T.sum((double)gg)));
        }
        bool ok = false, have_gn = false;
        for (int ls = 0; ls < cfg.max_ls; ++ls) {
            const double pt = team_objective<Noise>(T, nz, h, d, alpha, n, dx, lt, f, model);
            ++res.n_func_evals;
            if (pt <= phi0 + cfg.c1 * alpha * dphi0) {
                phi = pt;
                ok = true;
                break;
            }
            if (cfg.ls_fallback) {  // slope test at the trial point xt = h + alpha d
                for (int i = t0; i < n; i += ts) xt[i] = h[i] + alpha * (double)d[i];
                T.sync();
                team_gradient<Noise>(T, nz, xt, n, dx, lt, f, arc, ev, es, gn);
                Real sd = 0;
                for (int i = t0; i < n; i += ts) sd += gn[i] * d[i];
                const double dphia = T.sum((double)sd);
                ++res.n_func_evals;
                if (dphia >= kAwSigma * dphi0 && dphia <= (2.0 * kAwDelta - 1.0) * dphi0 &&
                    pt <= phi0 + kAwEps * fabs(phi0)) {
                    phi = pt;
                    ok = true;
                    have_gn = true;  // gn already holds the gradient at the new point
                    break;
                }
            }
            alpha *= cfg.ls_shrink;
        }
        if (!ok) {
            if (empty || ++ls_fail_streak > 2) {
                res.iterations = it;
                res.max_force = gmax;
                res.converged = 0;
                done = true;
                break;
            }
            if (threadIdx.x == 0) sh.nslots = 0;
            ++res.n_ls_restarts;
            T.sync();
            continue;
        }
        ls_fail_streak = 0;
        for (int i = t0; i < n; i += ts) h[i] += alpha * (double)d[i];  // lbfgs.h:243-244
        T.sync();
        if (!have_gn) team_gradient<Noise>(T, nz, h, n, dx, lt, f, arc, ev, es, gn);
        Real *sT = row(sh.stmp);
        Real *yT = row(sh.ytmp);
        Real syr = 0, ssr = 0, yyr = 0;
        for (int i = t0; i < n; i += ts) {  // lbfgs.h:250-261
            const Real s = (Real)(alpha * d[i]);
            const Real y = gn[i] - g[i];
            sT[i] = s;
            yT[i] = y;
            syr += s * y;
            ssr += s * s;
            yyr += y * y;
        }
        double sy = syr, ss = ssr, yy = yyr;
        T.sum3(sy, ss, yy);
        if (sy > cfg.curvature_eps * sqrt(ss * yy)) {  // lbfgs.h:262-279
            if (threadIdx.x == 0) {
                int row;
                if (sh.nslots < m) {
                    row = sh.nslots;
                } else {
                    row = sh.slots[0];
                    for (int k = 0; k + 1 < sh.nslots; ++k) sh.slots[k] = sh.slots[k + 1];
                    --sh.nslots;
                }
                int tmp = sh.sbuf[row];
                sh.sbuf[row] = sh.stmp;
                sh.stmp = tmp;
                tmp = sh.ybuf[row];
                sh.ybuf[row] = sh.ytmp;
                sh.ytmp = tmp;
                sh.rho[row] = 1.0 / sy;
                sh.slots[sh.nslots++] = row;
            }
            gamma = sy / yy;
        } else {
            ++res.n_curvature_skips;
        }
        T.sync();
        Real *tg = g;
        g = gn;
        gn = tg;
    }
    if (!done) {  // lbfgs.h:283-286
        double lm = 0.0;
        for (int i = t0; i < n; i += ts) lm = fmax(lm, fabs((double)g[i]));
        res.iterations = cfg.max_iter;
        res.max_force = T.max(lm);
        res.converged = 0;
    }
    return res;  // identical in every thread
}


// One CTA runs the whole solve (the single-line resident form and the
// ensemble's CTA per line).
template <class Noise, int BS, class Real = double>
__device__ qew_lbfgs_result lbfgs_block(const Noise &nz, double *__restrict__ h, const int n,
                                        const qew_params P, const LbfgsCfg cfg,
                                        const PrecondCoef pc, double *ws, size_t npad) {
    __shared__ double s_w[96];
    CtaTeam<BS> T{s_w};
    return lbfgs_team<Noise, CtaTeam<BS>, Real>(T, nz, h, n, P, cfg, pc, ws, npad);
}

size_t qew_lbfgs_resident_ws_doubles(int n, int m);
