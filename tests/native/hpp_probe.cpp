// Exercises the C++ face (include/qew_gpu.hpp) the way a reference caller
// would: device lines owned by the caller, the reference's signatures and
// exceptions. Prints one line per check; exit status 0 when all pass.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "qew_gpu.hpp"

using namespace qew::gpu;

static double *upload(const std::vector<double> &h) {
    double *d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(double)) != cudaSuccess) throw std::runtime_error("alloc");
    cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
    return d;
}
static std::vector<double> download(const double *d, int n) {
    std::vector<double> h(n);
    cudaMemcpy(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost);
    return h;
}
#define CHECK(cond, msg)                                  \
    do {                                                  \
        if (!(cond)) {                                    \
            std::printf("FAIL %s\n", msg);                \
            return 1;                                     \
        }                                                 \
        std::printf("ok %s\n", msg);                      \
    } while (0)

int main() {
    try {
        Context ctx(0);
        // lbfgs_minimize on a harmonic trough reaches the flat line at y0
        {
            const int n = 96;
            Noise well = Noise::harmonic_well(ctx, 2.0, 0.5);
            double *d = upload(std::vector<double>(n, 0.0));
            Params p;
            p.physical_size = n;
            LbfgsParams lp;
            lp.ftol = 1e-10;
            const LbfgsResult r = lbfgs_minimize(d, n, p, well, lp);
            const std::vector<double> h = download(d, n);
            double dev = 0;
            for (double v : h) dev = std::fmax(dev, std::fabs(v - 0.5));
            CHECK(r.converged && dev < 1e-8, "lbfgs_minimize");
            const double e = objective(d, n, p, well);
            CHECK(std::fabs(e) < 1e-12, "objective");
            FireParams fp;
            fp.dt_max = 0.1;
            fp.ftol = 1e-9;
            cudaMemcpy(d, std::vector<double>(n, 0.0).data(), n * sizeof(double),
                       cudaMemcpyHostToDevice);
            const FireResult f = fire_minimize(d, n, p, well, fp);
            CHECK(f.converged, "fire_minimize");
            cudaFree(d);
        }
        // rk_block: odd n throws std::invalid_argument, as the reference does
        {
            Noise wb = Noise::washboard(ctx, 0.1, 2 * M_PI);
            double *d = upload(std::vector<double>(17, 0.0));
            RkParams rp;
            rp.dstep = 0.01;
            rp.max_advance = 1.0;
            rp.runaway = 3.0;
            bool thrown = false;
            try {
                rk_block(d, 17, Params{17.0, 1.0, 0.0, Model::Linear}, wb, rp);
            } catch (const std::invalid_argument &) {
                thrown = true;
            }
            CHECK(thrown, "rk_block odd n throws std::invalid_argument");
            cudaFree(d);
        }
        // the drivers
        {
            Noise zero = Noise::zero(ctx);
            StaticConfig sc;
            sc.model = Model::Linear;
            sc.nx = 16;
            sc.ny = 8;
            sc.Lx = 1.0;
            sc.pinning_lengths_over_xi = {0.1, 1.0};
            sc.ftol = 1e-8;
            const std::vector<StaticProfile> prof = static_sweep(sc, zero);
            CHECK(prof.size() == 2 && prof[1].result.converged &&
                      std::fabs(prof[1].h[3] - 0.5) < 1e-9,
                  "static_sweep");
            DepinningConfig dc;
            dc.model = Model::Linear;
            dc.pinning_length_over_xi = 1.0;
            dc.nx = 8;
            dc.ny = 8;
            dc.f_step = 0.2;
            dc.f_max = 2.0;
            dc.rp.dstep = 0.01;
            dc.rp.max_advance = 1.0;
            dc.rp.runaway = 3.0;
            dc.rp.root_tol = 1e-11;
            dc.rp.sweep_tol = 1e-8;
            dc.rp.max_sweeps = 20000;
            Noise wb = Noise::washboard(ctx, 0.1, 2 * M_PI);
            const DepinningResult dr = depinning_ramp(dc, wb);
            const double fc = 0.1 * 2 * M_PI;
            CHECK(dr.f_c_upper_bound - dc.f_step <= fc && fc <= dr.f_c_upper_bound + 1e-9,
                  "depinning_ramp");
            DynamicConfig yc;
            yc.model = Model::Linear;
            yc.nx = 32;
            yc.ny = 8;
            yc.Lx = 1.0;
            yc.total_time = 20.0;
            const DynamicResult yr = dynamic_anneal(yc, zero);
            CHECK(!yr.snapshots.empty() && yr.dt > 0, "dynamic_anneal");
        }
        // a bad argument surfaces as qew::gpu::Error with the library's message
        {
            Noise zero = Noise::zero(ctx);
            bool thrown = false;
            try {
                FireParams fp;  // dt_max missing
                fire_minimize(nullptr, 8, Params{}, zero, fp);
            } catch (const Error &e) {
                thrown = e.status == QEW_ERR_INVALID;
            }
            CHECK(thrown, "Error carries the status");
        }
    } catch (const std::exception &e) {
        std::printf("FAIL exception: %s\n", e.what());
        return 1;
    }
    return 0;
}
