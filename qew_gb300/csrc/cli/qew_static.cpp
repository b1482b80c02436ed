// qew_static -- L-BFGS relaxation of a flat line at each pinning length, the
// executable of the reference's static run (executables/qew_static/main.cpp)
// with the same options, defaults, console lines and output keys, on the GPU.
// Added options: --lbfgs_m (history size), --analysis 1 (write ell, acf, q,
// psd beside each profile, as the reference's post-processing does),
// --field_file (a given field), --rows (unit-spacing rows), --device.
#include <cstdio>
#include <string>
#include <vector>

#include "qew_cli_common.h"

using namespace qew;

namespace {
const char *kUsage =
    "qew_static -- L-BFGS relaxation, sweep over pinning length (GPU).\n"
    "All options take a value.\n\n"
    "  --model           linear|arclength      (default arclength)\n"
    "  --amplitude       disorder amplitude U0  (default 1)\n"
    "  --xi              correlation length     (default 0.1)\n"
    "  --Lx --Ly         system size            (default 32, 1)\n"
    "  --nx --ny         resolution             (default 4096, 512)\n"
    "  --driving_force   external force         (default 0)\n"
    "  --pinning_lengths comma list of lambda_p/xi (default 0.01,0.1,1,10,100)\n"
    "  --ftol            L-BFGS tolerance       (default 1e-6)\n"
    "  --max_iter        L-BFGS iteration cap   (default 5000)\n"
    "  --seed            noise RNG seed         (default 1)\n"
    "  --output          output file            (default static_<model>.npz, .h5 with HDF5)\n"
    "  --lbfgs_m         L-BFGS history size    (default 8)\n"
    "  --analysis        1: add ell, acf, q, psd beside each profile (default 0)\n"
    "  --field_file      float64 .npy field, shape (nx, ny), instead of the seeded one\n"
    "  --rows            R rows at unit spacing: --ny R --Ly R\n"
    "  --device          CUDA device            (default 0)\n";

int run(int argc, char **argv) {
    cli::Options a(argc, argv);
    if (a.help) {
        std::fputs(kUsage, stdout);
        return 0;
    }
    qew_static_config cfg;
    qew_static_config_default(&cfg);
    const std::string model = a.text("model", "arclength");
    cfg.model = cli::parse_model(model);
    cfg.amplitude = a.real("amplitude", 1.0);
    cfg.xi = a.real("xi", 0.1);
    cfg.Lx = a.real("Lx", 32.0);
    cfg.Ly = a.real("Ly", 1.0);
    cfg.nx = a.integer("nx", 4096);
    cfg.ny = a.integer("ny", 512);
    cli::apply_rows(a, cfg.ny, cfg.Ly);
    const std::vector<double> file_field = cli::field_from_file(a, cfg.nx, cfg.ny);
    cfg.driving_force = a.real("driving_force", 0.0);
    const std::vector<double> ratios =
        a.real_list("pinning_lengths", {0.01, 0.1, 1.0, 10.0, 100.0});
    cfg.pinning_lengths_over_xi = ratios.data();
    cfg.n_pinning_lengths = (int)ratios.size();
    cfg.ftol = a.real("ftol", 1e-6);
    cfg.max_iter = a.integer("max_iter", 5000);
    const uint64_t seed = a.u64("seed", 1);
    const std::string fname = a.text("output", "static_" + model + default_suffix());
    cfg.lbfgs_m = a.integer("lbfgs_m", 8);
    const bool analysis = a.integer("analysis", 0) != 0;
    const int device = a.integer("device", 0);
    a.finish();
    std::unique_ptr<Sink> sink = open_sink(fname);

    cli::Gpu gpu(device);
    gpu.field_for(file_field, cfg.nx, cfg.ny, cfg.Lx, cfg.Ly, cfg.amplitude, cfg.xi, seed,
                  QEW_STORE_FP64);
    std::vector<qew_static_profile> prof(ratios.size());
    std::vector<double> h(ratios.size() * (size_t)cfg.nx);
    gpu.check(qew_static_sweep(gpu.ctx, gpu.field, &cfg, prof.data(), h.data()), "static_sweep");

    std::vector<StaticOut> out;
    std::vector<LineStats> stats(prof.size());
    for (size_t k = 0; k < prof.size(); ++k) {
        const qew_static_profile &p = prof[k];
        std::printf("lp/xi=%-6.3g lt=%-10.4g iters=%-7d max|F|=%.3e  %s\n",
                    p.pinning_length_over_xi, p.line_tension, p.result.iterations,
                    p.result.max_force, p.result.converged ? "converged" : "NOT converged");
        out.push_back(StaticOut{p.pinning_length_over_xi,
                                std::vector<double>(h.begin() + k * cfg.nx,
                                                    h.begin() + (k + 1) * cfg.nx)});
        if (analysis) {
            stats[k] = cli::line_stats(gpu, out.back().h, cfg.Lx);
            out.back().stats = &stats[k];
        }
    }
    write_static(*sink, cfg, out);
    sink->close();
    std::printf("wrote %s\n", fname.c_str());
    return 0;
}
}  // namespace

int main(int argc, char **argv) { return cli::guarded_main("qew_static", kUsage, run, argc, argv); }
