// qew_server.cu -- serving: continuous batching of mixed requests (static
// minimisation, annealed Langevin, depinning f_c) with admission by an HBM
// budget. No reference counterpart: the reference runs one simulation per
// process (the three executables).
//
// Requests enter a queue. Each of `max_inflight` workers owns a context on
// its own non-blocking CUDA stream; a worker admits the oldest admissible
// request as soon as its device-memory estimate fits in the budget left by
// the requests in flight (depinning requests, the long ones, hold at most
// half the workers), so requests arriving while others run are admitted as
// slots and memory free up and their kernels overlap on the device. Static
// requests on short lines go to a device-resident loop instead (lane_main). Every
// buffer of a request (its generated field, its line, its solver state)
// lives on the device and is allocated and released in its stream's order,
// so finishing one request never waits for the others. Every kernel involved
// is deterministic with a launch shape fixed by the request alone, so a
// request's result is the same whether it runs alone or in the mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "qew_internal.cuh"
#include "qew_lbfgs_internal.cuh"
#include "qew_rk_internal.cuh"
#include "qew_serve_lane.cuh"
#include "qew_vec.cuh"

extern "C" void qew_field_release_on(qew_field *f, cudaStream_t stream);

struct qew_server {
    int device = 0;
    double budget = 0;
    double used = 0;
    int max_inflight = 1;
    std::mutex mu;
    std::condition_variable cv;
    struct Job {
        uint64_t id;
        qew_request req;
        double t_submit;
        double est;
    };
    std::deque<Job> queue;       // requests for the worker threads
    std::deque<Job> lane_queue;  // static lines for the device-resident loop
    std::vector<qew_response> done;
    std::vector<std::thread> workers;
    int workers_running = 0;  // requests the workers are serving
    int depinning_running = 0;  // of which depinning requests
    StaticLane *lane = nullptr;
    int lane_max_n = 2048;
    std::thread lane_thread;
    uint64_t lane_served = 0;
    int running = 0;
    bool stop = false;
    uint64_t next_id = 1;
    std::chrono::steady_clock::time_point t0;
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

// Static requests on lines of at most lane_max_n points (default 2048, the
// length up to which one CTA per line beats a thread-block cluster for a
// request alone; at most kLaneCapN, which sizes the loop's workspace), at
// the lane's tolerance, go to the device-resident loop; the lane takes one
// persistent CTA per SM.
constexpr int kLaneCapN = QEW_LANE_CAP_N;
constexpr double kLaneFtol = 1e-8;
constexpr int kLaneWarpsPerSm = 16;

bool lane_request(const qew_server *s, const qew_request &r) {
    return s->lane && r.kind == QEW_REQ_STATIC && r.n <= s->lane_max_n && r.ftol == kLaneFtol;
}

// Device bytes a request holds at its peak: field generation (two FP64
// work arrays + FP64 and FP32 coefficients) plus line and solver state.
double request_bytes(const qew_request &r) {
    const double cells = (double)r.n * (double)r.rows;
    return cells * (8.0 * 2 + 8.0 + 4.0) + (double)r.n * 8.0 * 40.0 + (1 << 20);
}

// Relaxes h in place at the request's force by the static path: FP32 phase
// to 2e-5, then FP64 refinement to ftol, preconditioned, m = 10, on a
// thread-block cluster for long lines, else on one CTA.
qew_status relax_line(qew_ctx *ctx, const qew_request &r, qew_field *f, double *h, double ftol,
                      double driving_force, qew_lbfgs_result &res);

qew_status run_static(qew_ctx *ctx, const qew_request &r, qew_field *f, double *h,
                      qew_response &out) {
    QEW_CUDA(ctx, cudaMemsetAsync(h, 0, sizeof(double) * (size_t)r.n, ctx->stream));
    qew_lbfgs_result res;
    QEW_TRY(relax_line(ctx, r, f, h, r.ftol, r.driving_force, res));
    out.iterations = res.iterations;
    out.max_force = res.max_force;
    out.converged = res.converged;
    const qew_params p{(double)r.n, r.line_tension, r.driving_force, r.model};
    return qew_objective(ctx, f, h, r.n, &p, &out.value);
}

qew_status relax_line(qew_ctx *ctx, const qew_request &r, qew_field *f, double *h, double ftol,
                      double driving_force, qew_lbfgs_result &res) {
    qew_ensemble_line line;
    line.field = f;
    line.d_h = h;
    line.n = r.n;
    line.p = qew_params{(double)r.n, r.line_tension, driving_force, r.model};
    line.precond_shift = 0.5 / (r.xi * r.xi);  // 0.5 dx A / xi^2 (qew_runs.h:89-91), dx = A = 1
    qew_ensemble_params ep;
    qew_lbfgs_default_params(&ep.lbfgs);
    ep.lbfgs.m = 10;
    ep.lbfgs.ftol = ftol;
    ep.lbfgs.max_iter = 20000;
    ep.lbfgs.precondition = 1;
    ep.lbfgs.ls_fallback = 1;
    ep.ftol_fp32 = 2e-5;
    ep.max_iter_fp32 = 0;
    // a long line runs on a thread-block cluster (both phases), else on one CTA
    double *hp[1] = {h};
    const double shift[1] = {line.precond_shift};
    qew_lbfgs_params lp32 = ep.lbfgs;
    lp32.ftol = ep.ftol_fp32;
    qew_lbfgs_result r32{};
    qew_status cs = qew_lbfgs_cluster_lines(ctx, f, 1, hp, r.n, &line.p, shift, &lp32, &r32,
                                            QEW_PREC_FP32_SPLIT);
    if (cs == QEW_OK)
        cs = qew_lbfgs_cluster_lines(ctx, f, 1, hp, r.n, &line.p, shift, &ep.lbfgs, &res);
    if (cs == QEW_OK) {
        res.iterations += r32.iterations;
        res.n_func_evals += r32.n_func_evals;
    } else if (cs == QEW_ERR_UNSUPPORTED) {
        QEW_TRY(qew_ensemble_minimize(ctx, 1, &line, &ep, &res));
    } else {
        return cs;
    }
    return QEW_OK;
}

qew_status run_langevin(qew_ctx *ctx, const qew_request &r, qew_field *f, double *h,
                        qew_response &out) {
    std::vector<double> hv((size_t)r.n, 0.5 * r.rows);
    QEW_CUDA(ctx, cudaMemcpyAsync(h, hv.data(), sizeof(double) * hv.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    qew_langevin *lgv = nullptr;
    QEW_TRY(qew_langevin_create(ctx, r.n, r.seed + 1, &lgv));
    std::vector<double> drift((size_t)r.steps, r.dt), diff((size_t)r.steps,
                                                         std::sqrt(2.0 * r.temperature * r.dt));
    const qew_params p{(double)r.n, r.line_tension, r.driving_force, r.model};
    qew_status st = qew_langevin_run(lgv, f, h, &p, r.steps, drift.data(), diff.data(),
                                     QEW_PREC_FP32_SPLIT);
    qew_langevin_destroy(lgv);
    QEW_TRY(st);
    double sum;
    QEW_TRY((vec_reduce<SumF, 1, false>(ctx, r.n, SumF{h}, &sum)));
    out.value = sum / r.n;
    out.iterations = r.steps;
    out.converged = 1;
    return QEW_OK;
}

qew_status run_depinning(qew_ctx *ctx, const qew_request &r, qew_field *f, double *h,
                         qew_response &out) {
    if (r.n % 2) return qew_fail(ctx, QEW_ERR_ODD_LENGTH, "depinning request: odd n");
    std::vector<double> hv((size_t)r.n, 0.5 * r.rows);
    QEW_CUDA(ctx, cudaMemcpyAsync(h, hv.data(), sizeof(double) * hv.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    // The ramp starts from the line relaxed at f = 0 (a local minimum of the
    // energy, every site velocity within 1e-6), not from the flat line: from
    // there the first no-passing block blocks in a few sweeps, where from the
    // flat line it can need more sweeps than a request allows.
    {
        qew_request rl = r;
        rl.model = QEW_MODEL_LINEAR;
        qew_lbfgs_result rr;
        QEW_TRY(relax_line(ctx, rl, f, h, 1e-6, 0.0, rr));
    }
    // CLI defaults of qew_depinning (main.cpp:75-81) in cells: dstep 1/2,
    // max_advance Ly, runaway 2 Ly, unless the request caps them
    qew_rk_params rp{0.5, r.max_advance > 0 ? r.max_advance : (double)r.rows, 1e-10, 1e-8,
                     r.runaway > 0 ? r.runaway : 2.0 * r.rows, r.max_sweeps};
    qew_params p{(double)r.n, r.line_tension, 0.0, QEW_MODEL_LINEAR};
    double *hlo = nullptr;
    QEW_TRY(qew_alloc_async(ctx, (void **)&hlo, sizeof(double) * (size_t)r.n));
    double f_lo = -1, f_hi = -1;
    int blocks = 0;
    qew_status st = QEW_OK;
    for (int k = 0; (double)k * r.f_step <= r.f_max; ++k) {  // ramp, qew_runs.h:224-241
        p.driving_force = (double)k * r.f_step;
        qew_rk_result rr;
        st = qew_rk_block_resident(ctx, f, h, r.n, &p, &rp, QEW_PREC_FP32_SPLIT, &rr);
        ++blocks;
        if (st != QEW_OK) break;
        if (!rr.blocked) {
            f_hi = p.driving_force;
            break;
        }
        f_lo = p.driving_force;
        cudaMemcpyAsync(hlo, h, sizeof(double) * (size_t)r.n, cudaMemcpyDeviceToDevice, ctx->stream);
    }
    if (st == QEW_OK && f_lo >= 0 && f_hi >= 0) {
        double fc, a, b;
        int nb = 0;
        st = qew_depinning_bisect_prec(ctx, f, hlo, r.n, &p, &rp, f_lo, f_hi, r.bisect_rtol, 64,
                                       QEW_PREC_FP32_SPLIT, &fc, &a, &b, &nb);
        blocks += nb;
        out.value = fc;
        out.converged = 1;
        cudaMemcpyAsync(h, hlo, sizeof(double) * (size_t)r.n, cudaMemcpyDeviceToDevice, ctx->stream);
    } else {
        out.value = f_hi;  // -1: no bracket within f_max
        out.converged = 0;
    }
    out.iterations = blocks;
    qew_free_async(hlo, ctx->stream);
    return st;
}

// The queued request a worker takes next, or -1: the oldest request whose
// device-memory estimate fits the budget left (or the first when nothing
// runs), where a depinning request (minutes of sweeps for a long line) is
// admissible only while depinning requests hold fewer than half the workers,
// so that short requests always find a worker. Called with s->mu held.
int pick_job(const qew_server *s) {
    const int depin_cap = std::max(1, s->max_inflight / 2);
    for (size_t k = 0; k < s->queue.size(); ++k) {
        const qew_server::Job &j = s->queue[k];
        if (j.req.kind == QEW_REQ_DEPINNING && s->depinning_running >= depin_cap) continue;
        if (s->used + j.est <= s->budget || s->used == 0) return (int)k;
        return -1;  // the oldest admissible request waits for memory: keep the order
    }
    return -1;
}

void worker_main(qew_server *s) {
    cudaSetDevice(s->device);
    qew_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    const bool ok = qew_ctx_create(s->device, &ctx) == QEW_OK &&
                    cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) {
        qew_ctx_set_stream(ctx, stream);
        // Langevin runs keep one grid barrier per step in the workers, without
        // tuning: a blocked run's cooperative grid, with its shared-memory
        // regions, has to find room beside the other requests' kernels at
        // launch, and a tuning probe times the other requests (the serving
        // mix measured p50 26.9-36.8 s against 4.4 s at 100 req/s with them).
        qew_ctx_force_tune_candidate(ctx, QEW_TUNE_LANGEVIN_RUN, 0);
    }
    // Persistent kernels of concurrent requests share the SMs: a request's
    // cooperative grids take at most its share of the GPU's warp slots (64 per
    // SM, less the static loop's), split among the requests the workers serve
    // when it starts, never less than four warps per SM. (Every launch shape
    // gives the same results, so the share changes no result.)
    const int warps = s->lane ? 64 - kLaneWarpsPerSm : 64;
    for (;;) {
        qew_server::Job job;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            int k = -1;
            s->cv.wait(lk, [&] { return s->stop || (k = pick_job(s)) >= 0; });
            if (s->stop && (s->queue.empty() || k < 0)) break;
            job = s->queue[(size_t)k];
            s->queue.erase(s->queue.begin() + k);
            s->used += job.est;
            ++s->running;
            ++s->workers_running;
            if (job.req.kind == QEW_REQ_DEPINNING) ++s->depinning_running;
            if (ctx)
                ctx->warp_cap = std::max(4 * ctx->num_sms,
                                         warps * ctx->num_sms / std::max(1, s->workers_running));
        }
        qew_response out{};
        out.id = job.id;
        out.kind = job.req.kind;
        out.t_submit = job.t_submit;
        out.t_start = s->now();
        qew_status st = ok ? QEW_OK : QEW_ERR_CUDA;
        qew_field *f = nullptr;
        double *h = nullptr;
        const qew_request &r = job.req;
        if (st == QEW_OK) {
            // FP64 for the static solves (and a depinning request's relaxation)
            const int store = (r.kind == QEW_REQ_LANGEVIN) ? QEW_STORE_FP32
                                                           : (QEW_STORE_FP64 | QEW_STORE_FP32);
            st = qew_field_create_generated(ctx, r.n, r.rows, (double)r.n, (double)r.rows, 1.0,
                                            r.xi, r.xi, r.seed, store, &f);
        }
        if (st == QEW_OK) st = qew_alloc_async(ctx, (void **)&h, sizeof(double) * (size_t)r.n);
        if (st == QEW_OK) {
            if (r.kind == QEW_REQ_STATIC)
                st = run_static(ctx, r, f, h, out);
            else if (r.kind == QEW_REQ_LANGEVIN)
                st = run_langevin(ctx, r, f, h, out);
            else if (r.kind == QEW_REQ_DEPINNING)
                st = run_depinning(ctx, r, f, h, out);
            else
                st = QEW_ERR_INVALID;
        }
        if (st == QEW_OK && r.h_out)
            if (cudaMemcpyAsync(r.h_out, h, sizeof(double) * (size_t)r.n, cudaMemcpyDeviceToHost,
                                stream) != cudaSuccess)
                st = QEW_ERR_CUDA;
        if (ctx) {
            qew_free_async(h, stream);
            qew_field_release_on(f, stream);
            if (cudaStreamSynchronize(stream) != cudaSuccess && st == QEW_OK) st = QEW_ERR_CUDA;
        }
        out.status = st;
        out.t_end = s->now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->used -= job.est;
            --s->running;
            --s->workers_running;
            if (job.req.kind == QEW_REQ_DEPINNING) --s->depinning_running;
            s->done.push_back(out);
        }
        s->cv.notify_all();
    }
    if (ctx) qew_ctx_destroy(ctx);
    if (stream) cudaStreamDestroy(stream);
}

// The device-resident loop's host side: builds each admitted static
// request's field and line on the device, publishes the job to the lane's
// ring (the persistent grid picks it up while it runs), relaunches the grid
// when it has left with jobs unclaimed, and collects finished jobs.
void lane_main(qew_server *s) {
    cudaSetDevice(s->device);
    qew_ctx *ctx = nullptr;
    cudaStream_t aux = nullptr;
    const bool ok = qew_ctx_create(s->device, &ctx) == QEW_OK &&
                    cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) qew_ctx_set_stream(ctx, aux);
    struct Flight {
        unsigned int k;
        qew_server::Job job;
        qew_field *f;
        double *h;
        double t_start;
    };
    std::deque<Flight> flight;
    auto finish = [&](const qew_server::Job &job, double t_start, qew_status st,
                      const qew_response *r) {
        qew_response out = r ? *r : qew_response{};
        out.id = job.id;
        out.kind = job.req.kind;
        out.t_submit = job.t_submit;
        out.t_start = t_start;
        out.status = st;
        out.t_end = s->now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->used -= job.est;
            --s->running;
            ++s->lane_served;
            s->done.push_back(out);
        }
        s->cv.notify_all();
    };
    for (;;) {
        bool busy = false;
        while ((int)flight.size() < kLaneRing - 1) {  // admit
            qew_server::Job job;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                if (s->lane_queue.empty()) break;
                const double est = s->lane_queue.front().est;
                if (!(s->used + est <= s->budget || s->used == 0)) break;
                job = s->lane_queue.front();
                s->lane_queue.pop_front();
                s->used += est;
                ++s->running;
            }
            busy = true;
            const double t_start = s->now();
            const qew_request &r = job.req;
            qew_field *f = nullptr;
            double *h = nullptr;
            qew_status st = ok ? QEW_OK : QEW_ERR_CUDA;
            if (st == QEW_OK)
                st = qew_field_create_generated(ctx, r.n, r.rows, (double)r.n, (double)r.rows,
                                                1.0, r.xi, r.xi, r.seed,
                                                QEW_STORE_FP64 | QEW_STORE_FP32, &f);
            if (st == QEW_OK) st = qew_alloc_async(ctx, (void **)&h, sizeof(double) * (size_t)r.n);
            if (st == QEW_OK && (cudaMemsetAsync(h, 0, sizeof(double) * (size_t)r.n, aux) !=
                                     cudaSuccess ||
                                 cudaStreamSynchronize(aux) != cudaSuccess))
                st = QEW_ERR_CUDA;  // the line is ready before the grid may read it
            unsigned int k = 0;
            if (st == QEW_OK) {
                const qew_params p{(double)r.n, r.line_tension, r.driving_force, r.model};
                // shift 0.5 dx A / xi^2 (qew_runs.h:89-91), dx = A = 1
                st = qew_lane_publish(s->lane, f, h, r.n, &p, 0.5 / (r.xi * r.xi), &k);
            }
            if (st != QEW_OK) {
                if (h) qew_free_async(h, aux);
                if (f) qew_field_release_on(f, aux);
                cudaStreamSynchronize(aux);
                finish(job, t_start, st, nullptr);
                continue;
            }
            flight.push_back(Flight{k, job, f, h, t_start});
        }
        if (ok && !flight.empty() && qew_lane_pump(s->lane, aux) != QEW_OK) {
            for (auto &fl : flight) finish(fl.job, fl.t_start, QEW_ERR_CUDA, nullptr);
            flight.clear();  // their memory stays with the failed grid
        }
        for (auto it = flight.begin(); it != flight.end();) {  // collect
            qew_lbfgs_result res;
            if (!qew_lane_done(s->lane, it->k, &res)) {
                ++it;
                continue;
            }
            busy = true;
            const qew_request &r = it->job.req;
            qew_response out{};
            out.iterations = res.iterations;
            out.max_force = res.max_force;
            out.converged = res.converged;
            const qew_params p{(double)r.n, r.line_tension, r.driving_force, r.model};
            qew_status st = qew_objective(ctx, it->f, it->h, r.n, &p, &out.value);
            if (st == QEW_OK && r.h_out &&
                cudaMemcpyAsync(r.h_out, it->h, sizeof(double) * (size_t)r.n,
                                cudaMemcpyDeviceToHost, aux) != cudaSuccess)
                st = QEW_ERR_CUDA;
            qew_free_async(it->h, aux);
            qew_field_release_on(it->f, aux);
            if (cudaStreamSynchronize(aux) != cudaSuccess && st == QEW_OK) st = QEW_ERR_CUDA;
            finish(it->job, it->t_start, st, &out);
            it = flight.erase(it);
        }
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->lane_queue.empty() && flight.empty()) break;
            if (flight.empty() && s->lane_queue.empty()) {
                s->cv.wait(lk, [&] { return s->stop || !s->lane_queue.empty(); });
                continue;
            }
        }
        if (!busy) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (ctx) qew_ctx_destroy(ctx);
    if (aux) cudaStreamDestroy(aux);
}

}  // namespace

extern "C" {

qew_status qew_server_create(int device, double hbm_budget_bytes, int max_inflight,
                             qew_server **out) {
    if (!out || max_inflight < 1 || max_inflight > 1024 || !(hbm_budget_bytes > 0))
        return QEW_ERR_INVALID;
    qew_server *s = new (std::nothrow) qew_server();
    if (!s) return QEW_ERR_NOMEM;
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_inflight = max_inflight;
    s->t0 = std::chrono::steady_clock::now();
    {
        int sms = 0, prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess) {
            qew_lbfgs_params lp;
            qew_lbfgs_default_params(&lp);
            lp.m = 10;
            lp.ftol = kLaneFtol;
            lp.max_iter = 20000;
            lp.precondition = 1;
            lp.ls_fallback = 1;
            // the same settings as the worker path's static requests
            if (qew_lane_create(device, kLaneCapN, &lp, 2e-5, sms, &s->lane) != QEW_OK)
                s->lane = nullptr;  // static requests then all take the worker path
        }
        cudaGetLastError();
        cudaSetDevice(prev);
    }
    try {
        if (s->lane) s->lane_thread = std::thread(lane_main, s);
        for (int k = 0; k < max_inflight; ++k) s->workers.emplace_back(worker_main, s);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv.notify_all();
        for (auto &t : s->workers) t.join();
        if (s->lane_thread.joinable()) s->lane_thread.join();
        qew_lane_destroy(s->lane);
        delete s;
        return QEW_ERR_NOMEM;
    }
    *out = s;
    return QEW_OK;
}

double qew_server_clock(const qew_server *s) { return s ? s->now() : 0.0; }

qew_status qew_server_lane_stats(qew_server *s, uint64_t *served, uint64_t *launches) {
    if (!s) return QEW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (served) *served = s->lane_served;
    if (launches) *launches = qew_lane_launches(s->lane);
    return s->lane ? QEW_OK : QEW_ERR_UNSUPPORTED;
}

qew_status qew_server_set_lane_limit(qew_server *s, int max_n) {
    if (!s || max_n < 0 || max_n > kLaneCapN) return QEW_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lane_max_n = max_n;
    return QEW_OK;
}

qew_status qew_server_submit(qew_server *s, const qew_request *req, uint64_t *id) {
    if (!s || !req || req->n < 2 || req->rows < 4 || !(req->xi >= 0) ||
        req->kind < QEW_REQ_STATIC || req->kind > QEW_REQ_DEPINNING)
        return QEW_ERR_INVALID;
    if (req->kind == QEW_REQ_LANGEVIN && (req->steps < 0 || !(req->dt > 0) || req->temperature < 0))
        return QEW_ERR_INVALID;
    if (req->kind == QEW_REQ_DEPINNING &&
        (req->n % 2 || !(req->f_step > 0) || req->max_sweeps < 1 || !(req->bisect_rtol > 0) ||
         !std::isfinite(req->f_max) || req->f_max / req->f_step > 1e9))
        return QEW_ERR_INVALID;  // the ramp's force count is bounded as qew_depinning_ramp's
    const double est = request_bytes(*req);
    if (est > s->budget) return QEW_ERR_NOMEM;  // could never be admitted
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return QEW_ERR_INVALID;
        qew_server::Job j{s->next_id++, *req, s->now(), est};
        if (id) *id = j.id;
        if (lane_request(s, *req))
            s->lane_queue.push_back(j);
        else
            s->queue.push_back(j);
    }
    s->cv.notify_all();
    return QEW_OK;
}

int qew_server_poll(qew_server *s, qew_response *out, int max) {
    if (!s || !out || max < 1) return 0;
    std::lock_guard<std::mutex> lk(s->mu);
    const int k = std::min<int>(max, (int)s->done.size());
    std::copy(s->done.begin(), s->done.begin() + k, out);
    s->done.erase(s->done.begin(), s->done.begin() + k);
    return k;
}

qew_status qew_server_drain(qew_server *s, double timeout_s) {
    if (!s) return QEW_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return s->queue.empty() && s->lane_queue.empty() && s->running == 0;
    });
    return ok ? QEW_OK : QEW_ERR_TIMEOUT;
}

qew_status qew_server_destroy(qew_server *s) {
    if (!s) return QEW_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->queue.clear();
        s->lane_queue.clear();
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto &t : s->workers) t.join();
    if (s->lane_thread.joinable()) s->lane_thread.join();
    qew_lane_destroy(s->lane);
    delete s;
    return QEW_OK;
}

}  // extern "C"
