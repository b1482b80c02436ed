/*
 * qew_gpu.hpp -- header-only C++ face of the C ABI (qew_gpu.h, qew_runs.h):
 * the reference's types and call signatures (qew_model.h, lbfgs.h,
 * dynamics.h, rosso_krauth.h, fire.h, qew_runs.h) with its error behaviour
 * restored -- std::invalid_argument where the reference throws it (odd n in
 * rk_block), qew::gpu::Error for failures of the GPU path -- and RAII
 * handles. Lines are device pointers plus a length (what View1D::data() and
 * extent(0) give on a CUDA build); the Noise argument of every call is a
 * qew::gpu::Noise handle, which also carries the context the call runs on.
 *
 * No reference counterpart beyond the signatures it mirrors; nothing here
 * computes, every call goes to the CUDA library.
 */
#ifndef QEW_GPU_HPP
#define QEW_GPU_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "qew_gpu.h"
#include "qew_runs.h"

namespace qew {
namespace gpu {

// ------------------------------------------------------------------ errors
class Error : public std::runtime_error {
  public:
    Error(qew_status s, const std::string &what) : std::runtime_error(what), status(s) {}
    qew_status status;
};

inline void check(qew_status s, const qew_ctx *ctx, const char *what) {
    if (s == QEW_OK) return;
    std::string msg = std::string(what) + ": ";
    msg += (ctx && qew_last_error(ctx)[0]) ? qew_last_error(ctx) : qew_status_string(s);
    if (s == QEW_ERR_ODD_LENGTH) throw std::invalid_argument(msg);  // rosso_krauth.h:134-136
    throw Error(s, msg);
}

// ------------------------------------------------------------------- types
enum class Model { Linear = QEW_MODEL_LINEAR, Arclength = QEW_MODEL_ARCLENGTH };  // qew_model.h:20

struct Params {  // qew_model.h:22-27
    double physical_size = 1.0;
    double line_tension = 1.0;
    double driving_force = 0.0;
    Model model = Model::Linear;
    qew_params c() const {
        return qew_params{physical_size, line_tension, driving_force, (int)model};
    }
};

struct LbfgsParams {  // lbfgs.h:32-52
    int m = 8;
    double ftol = 1e-6;
    int max_iter = 10000;
    double c1 = 1e-4;
    double ls_shrink = 0.5;
    int max_ls = 30;
    double curvature_eps = 1e-12;
    bool precondition = false;
    double precond_shift = 0.0;
    bool ls_fallback = false;  // added: approximate-Wolfe fallback (qew_gpu.h)
    qew_lbfgs_params c() const {
        return qew_lbfgs_params{m,      ftol,          max_iter,          c1,
                                ls_shrink, max_ls,     curvature_eps,     precondition ? 1 : 0,
                                precond_shift, ls_fallback ? 1 : 0};
    }
};

struct LbfgsResult {  // lbfgs.h:54-61
    int iterations = 0;
    double max_force = 0.0;
    bool converged = false;
    long n_func_evals = 0;
    long n_curvature_skips = 0;
    long n_ls_restarts = 0;
};

inline LbfgsResult from_c(const qew_lbfgs_result &r) {
    return LbfgsResult{r.iterations,   r.max_force,         r.converged != 0,
                       r.n_func_evals, r.n_curvature_skips, r.n_ls_restarts};
}

struct RkParams {  // rosso_krauth.h:34-41
    double dstep = 0.0;
    double max_advance = 0.0;
    double root_tol = 1e-10;
    double sweep_tol = 1e-9;
    double runaway = 0.0;
    int max_sweeps = 200000;
    qew_rk_params c() const {
        return qew_rk_params{dstep, max_advance, root_tol, sweep_tol, runaway, max_sweeps};
    }
};

struct RkResult {  // rosso_krauth.h:43-49
    bool blocked = false;
    bool runaway = false;
    int sweeps = 0;
    double total_advance = 0.0;
    double mean_h = 0.0;
};

inline RkResult from_c(const qew_rk_result &r) {
    return RkResult{r.blocked != 0, r.runaway != 0, r.sweeps, r.total_advance, r.mean_h};
}

struct FireParams {  // fire.h:21-31
    double dt_max = 0.0;
    double dt_init = 0.0;
    double ftol = 1e-6;
    int max_iter = 100000;
    int n_min = 5;
    double f_inc = 1.1;
    double f_dec = 0.5;
    double alpha_start = 0.1;
    double f_alpha = 0.99;
    qew_fire_params c() const {
        return qew_fire_params{dt_max, dt_init, ftol,        max_iter, n_min,
                               f_inc,  f_dec,   alpha_start, f_alpha};
    }
};

struct FireResult {  // fire.h:33-37
    int iterations = 0;
    double max_force = 0.0;
    bool converged = false;
};

// ----------------------------------------------------------------- handles
class Context {
  public:
    explicit Context(int device = 0) { check(qew_ctx_create(device, &ctx_), nullptr, "context"); }
    ~Context() {
        if (ctx_) qew_ctx_destroy(ctx_);
    }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    Context(Context &&o) noexcept : ctx_(std::exchange(o.ctx_, nullptr)) {}
    qew_ctx *get() const { return ctx_; }
    void set_stream(void *cuda_stream) {
        check(qew_ctx_set_stream(ctx_, cuda_stream), ctx_, "set_stream");
    }
    void synchronize() { check(qew_ctx_synchronize(ctx_), ctx_, "synchronize"); }

  private:
    qew_ctx *ctx_ = nullptr;
};

// The pinning potential: a B-spline field (FilteredNoise) or one of the
// reference tests' analytic potentials. Keeps the context it was made on.
class Noise {
  public:
    // FilteredNoise(field, nx, ny, Lx, Ly) (filtered_noise.h:187-189);
    // h_field is the host array field[i * ny + j].
    static Noise filtered(Context &ctx, const double *h_field, int nx, int ny, double Lx,
                          double Ly, int store = QEW_STORE_FP64) {
        Noise nz(ctx);
        check(qew_field_create_from_host(ctx.get(), h_field, nx, ny, Lx, Ly, store, &nz.f_),
              ctx.get(), "FilteredNoise");
        return nz;
    }
    // FilteredNoise(nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed) (filtered_noise.h:183-185)
    static Noise seeded(Context &ctx, int nx, int ny, double Lx, double Ly, double amplitude,
                        double xi_x, double xi_y, std::uint64_t seed, int store = QEW_STORE_FP64) {
        Noise nz(ctx);
        check(qew_field_create_seeded(ctx.get(), nx, ny, Lx, Ly, amplitude, xi_x, xi_y, seed,
                                      store, &nz.f_),
              ctx.get(), "FilteredNoise");
        return nz;
    }
    static Noise zero(Context &ctx) { return analytic(ctx, QEW_FIELD_ZERO); }
    static Noise constant(Context &ctx, double v0) { return analytic(ctx, QEW_FIELD_CONST, v0); }
    static Noise harmonic_well(Context &ctx, double k, double y0) {
        return analytic(ctx, QEW_FIELD_HARMONIC, k, y0);
    }
    static Noise washboard(Context &ctx, double A, double k) {
        return analytic(ctx, QEW_FIELD_WASHBOARD, A, k);
    }
    ~Noise() {
        if (f_) qew_field_destroy(f_);
    }
    Noise(const Noise &) = delete;
    Noise &operator=(const Noise &) = delete;
    Noise(Noise &&o) noexcept : ctx_(o.ctx_), f_(std::exchange(o.f_, nullptr)) {}
    qew_ctx *ctx() const { return ctx_; }
    const qew_field *field() const { return f_; }

  private:
    explicit Noise(Context &ctx) : ctx_(ctx.get()) {}
    static Noise analytic(Context &ctx, int kind, double p0 = 0, double p1 = 0, double p2 = 0) {
        Noise nz(ctx);
        check(qew_field_create_analytic(ctx.get(), kind, p0, p1, p2, &nz.f_), ctx.get(), "noise");
        return nz;
    }
    qew_ctx *ctx_ = nullptr;
    qew_field *f_ = nullptr;
};

// ---------------------------------------------------------- operator calls
// objective(h, p, noise), qew_model.h:102-109
inline double objective(const double *d_h, int n, const Params &p, const Noise &nz) {
    const qew_params c = p.c();
    double e = 0.0;
    check(qew_objective(nz.ctx(), nz.field(), d_h, n, &c, &e), nz.ctx(), "objective");
    return e;
}
// objective(x0, d, alpha, p, noise), qew_model.h:112-119
inline double objective(const double *d_x0, const double *d_d, double alpha, int n,
                        const Params &p, const Noise &nz) {
    const qew_params c = p.c();
    double e = 0.0;
    check(qew_objective_trial(nz.ctx(), nz.field(), d_x0, d_d, alpha, n, &c, &e), nz.ctx(),
          "objective");
    return e;
}
// gradient(h, p, noise, grad), qew_model.h:149-201
inline void gradient(const double *d_h, int n, const Params &p, const Noise &nz, double *d_grad) {
    const qew_params c = p.c();
    check(qew_gradient(nz.ctx(), nz.field(), d_h, n, &c, d_grad), nz.ctx(), "gradient");
}
// lbfgs_minimize(h, p, noise, lp), lbfgs.h:94-96
inline LbfgsResult lbfgs_minimize(double *d_h, int n, const Params &p, const Noise &nz,
                                  const LbfgsParams &lp = LbfgsParams()) {
    const qew_params c = p.c();
    const qew_lbfgs_params l = lp.c();
    qew_lbfgs_result r{};
    check(qew_lbfgs_minimize(nz.ctx(), nz.field(), d_h, n, &c, &l, &r), nz.ctx(),
          "lbfgs_minimize");
    return from_c(r);
}
// fire_minimize(h, p, noise, fp), fire.h:41-131
inline FireResult fire_minimize(double *d_h, int n, const Params &p, const Noise &nz,
                                const FireParams &fp) {
    const qew_params c = p.c();
    const qew_fire_params f = fp.c();
    qew_fire_result r{};
    check(qew_fire_minimize(nz.ctx(), nz.field(), d_h, n, &c, &f, &r), nz.ctx(), "fire_minimize");
    return FireResult{r.iterations, r.max_force, r.converged != 0};
}
// rk_site_velocity of every site, rosso_krauth.h:51-82
inline void rk_site_velocity(const double *d_h, int n, const Params &p, const Noise &nz,
                             double *d_vel) {
    const qew_params c = p.c();
    check(qew_rk_site_velocity(nz.ctx(), nz.field(), d_h, n, &c, d_vel), nz.ctx(),
          "rk_site_velocity");
}
// rk_block(h, p, noise, rp), rosso_krauth.h:128-194: std::invalid_argument on odd n
inline RkResult rk_block(double *d_h, int n, const Params &p, const Noise &nz,
                         const RkParams &rp) {
    const qew_params c = p.c();
    const qew_rk_params r = rp.c();
    qew_rk_result o{};
    check(qew_rk_block(nz.ctx(), nz.field(), d_h, n, &c, &r, &o), nz.ctx(), "rk_block");
    return from_c(o);
}

// LangevinDynamics(n, seed) and step(h, p, noise, drift, diff), dynamics.h:27-70
class LangevinDynamics {
  public:
    LangevinDynamics(Context &ctx, int n, std::uint64_t seed) : ctx_(ctx.get()) {
        check(qew_langevin_create(ctx.get(), n, seed, &l_), ctx.get(), "LangevinDynamics");
    }
    ~LangevinDynamics() {
        if (l_) qew_langevin_destroy(l_);
    }
    LangevinDynamics(const LangevinDynamics &) = delete;
    LangevinDynamics &operator=(const LangevinDynamics &) = delete;
    void step(double *d_h, const Params &p, const Noise &nz, double drift, double diff) {
        const qew_params c = p.c();
        check(qew_langevin_step(l_, nz.field(), d_h, &c, drift, diff), ctx_, "step");
    }

  private:
    qew_ctx *ctx_ = nullptr;
    qew_langevin *l_ = nullptr;
};

// ----------------------------------------------------------------- drivers
// StaticConfig / StaticProfile / static_sweep, qew_runs.h:48-102
struct StaticConfig {
    Model model = Model::Arclength;
    double amplitude = 1.0;
    double xi = 0.1;
    double Lx = 32.0;
    double Ly = 1.0;
    int nx = 4096;
    int ny = 512;
    double driving_force = 0.0;
    std::vector<double> pinning_lengths_over_xi = {0.01, 0.1, 1.0, 10.0, 100.0};
    double ftol = 1e-6;
    int max_iter = 5000;
};

struct StaticProfile {
    double pinning_length_over_xi = 0;
    double line_tension = 0;
    std::vector<double> h;
    LbfgsResult result;
};

inline std::vector<StaticProfile> static_sweep(const StaticConfig &c, const Noise &nz) {
    qew_static_config q;
    qew_static_config_default(&q);
    q.model = (int)c.model;
    q.amplitude = c.amplitude;
    q.xi = c.xi;
    q.Lx = c.Lx;
    q.Ly = c.Ly;
    q.nx = c.nx;
    q.ny = c.ny;
    q.driving_force = c.driving_force;
    q.pinning_lengths_over_xi = c.pinning_lengths_over_xi.data();
    q.n_pinning_lengths = (int)c.pinning_lengths_over_xi.size();
    q.ftol = c.ftol;
    q.max_iter = c.max_iter;
    std::vector<qew_static_profile> pr(c.pinning_lengths_over_xi.size());
    std::vector<double> h(pr.size() * (size_t)c.nx);
    check(qew_static_sweep(nz.ctx(), nz.field(), &q, pr.data(), h.data()), nz.ctx(),
          "static_sweep");
    std::vector<StaticProfile> out(pr.size());
    for (size_t k = 0; k < pr.size(); ++k) {
        out[k].pinning_length_over_xi = pr[k].pinning_length_over_xi;
        out[k].line_tension = pr[k].line_tension;
        out[k].h.assign(h.begin() + k * c.nx, h.begin() + (k + 1) * c.nx);
        out[k].result = from_c(pr[k].result);
    }
    return out;
}

// DynamicConfig / DynamicResult / dynamic_anneal, qew_runs.h:107-177
struct DynamicConfig {
    Model model = Model::Arclength;
    double amplitude = 1.0;
    double xi = 0.1;
    double pinning_length_over_xi = 0.1;
    double driving_force = 0.0;
    double Lx = 2.0;
    double Ly = 1.0;
    int nx = 2048;
    int ny = 1024;
    std::uint64_t seed = 1;
    double tau = 1.0;
    double tl_start = 0.01;
    double tl_end = 0.0001;
    double total_time = 1000.0;
};

struct DynamicSnapshot {
    double t = 0;
    std::vector<double> h;
};

struct DynamicResult {
    double dt = 0;
    double total_time = 0;
    double line_tension = 0;
    std::vector<DynamicSnapshot> snapshots;
};

inline DynamicResult dynamic_anneal(const DynamicConfig &c, const Noise &nz) {
    qew_dynamic_config q;
    qew_dynamic_config_default(&q);
    q.model = (int)c.model;
    q.amplitude = c.amplitude;
    q.xi = c.xi;
    q.pinning_length_over_xi = c.pinning_length_over_xi;
    q.driving_force = c.driving_force;
    q.Lx = c.Lx;
    q.Ly = c.Ly;
    q.nx = c.nx;
    q.ny = c.ny;
    q.seed = c.seed;
    q.tau = c.tau;
    q.tl_start = c.tl_start;
    q.tl_end = c.tl_end;
    q.total_time = c.total_time;
    DynamicResult out;
    auto on = [](void *user, double t, const double *h, int n) {
        static_cast<DynamicResult *>(user)->snapshots.push_back(
            DynamicSnapshot{t, std::vector<double>(h, h + n)});
    };
    qew_dynamic_result r{};
    check(qew_dynamic_anneal(nz.ctx(), nz.field(), &q, on, &out, &r), nz.ctx(), "dynamic_anneal");
    out.dt = r.dt;
    out.total_time = r.total_time;
    out.line_tension = r.line_tension;
    return out;
}

// DepinningConfig / DepinningResult / depinning_ramp, qew_runs.h:182-243
struct DepinningConfig {
    Model model = Model::Arclength;
    double amplitude = 1.0;
    double xi = 0.1;
    double pinning_length_over_xi = 5.0;
    double Lx = 8.0;
    double Ly = 1.0;
    int nx = 1024;
    int ny = 256;
    double f_step = 1.0;
    double f_max = 40.0;
    RkParams rp;
};

struct DepinningStep {
    double f = 0;
    RkResult result;
    std::vector<double> h;  // blocked steps only
};

struct DepinningResult {
    double line_tension = 0;
    double f_c_upper_bound = -1;
    std::vector<DepinningStep> steps;
};

inline DepinningResult depinning_ramp(const DepinningConfig &c, const Noise &nz) {
    qew_depinning_config q;
    qew_depinning_config_default(&q);
    q.model = (int)c.model;
    q.amplitude = c.amplitude;
    q.xi = c.xi;
    q.pinning_length_over_xi = c.pinning_length_over_xi;
    q.Lx = c.Lx;
    q.Ly = c.Ly;
    q.nx = c.nx;
    q.ny = c.ny;
    q.f_step = c.f_step;
    q.f_max = c.f_max;
    q.rp = c.rp.c();
    DepinningResult out;
    auto on = [](void *user, const qew_depinning_step *st, const double *h, int n) {
        DepinningStep s;
        s.f = st->f;
        s.result = from_c(st->result);
        if (h) s.h.assign(h, h + n);
        static_cast<DepinningResult *>(user)->steps.push_back(std::move(s));
    };
    qew_depinning_result r{};
    check(qew_depinning_ramp(nz.ctx(), nz.field(), &q, on, &out, &r), nz.ctx(), "depinning_ramp");
    out.line_tension = r.line_tension;
    out.f_c_upper_bound = r.f_c_upper_bound;
    return out;
}

}  // namespace gpu
}  // namespace qew

#endif  // QEW_GPU_HPP
