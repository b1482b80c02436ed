// qew_dynamic -- annealed overdamped Langevin dynamics, the executable of the
// reference's dynamic run (executables/qew_dynamic/main.cpp) with the same
// options, defaults, console lines and output keys, on the GPU. Added
// options: --dt (explicit timestep), --precision fp64|fp32split, --analysis 1
// (ell, acf, q, psd beside each snapshot), --field_file (a given field),
// --rows (unit-spacing rows), --device.
#include <cstdio>
#include <string>
#include <vector>

#include "qew_cli_common.h"

using namespace qew;

namespace {
const char *kUsage =
    "qew_dynamic -- annealed overdamped Langevin dynamics (GPU).\n"
    "All options take a value.\n\n"
    "  --model           linear|arclength      (default arclength)\n"
    "  --amplitude       disorder amplitude U0  (default 1)\n"
    "  --xi              correlation length     (default 0.1)\n"
    "  --pinning_length  lambda_p/xi            (default 0.1)\n"
    "  --driving_force   external force         (default 0)\n"
    "  --Lx --Ly         system size            (default 2, 1)\n"
    "  --nx --ny         resolution             (default 2048, 1024)\n"
    "  --tau             damping time           (default 1)\n"
    "  --tl_start        anneal thermal length, start (default 0.01)\n"
    "  --tl_end          anneal thermal length, end   (default 0.0001)\n"
    "  --total_time      integration time       (default 1000)\n"
    "  --seed            noise/RNG seed         (default 1)\n"
    "  --output          output file            (default dynamic_<model>.npz, .h5 with HDF5)\n"
    "  --dt              timestep               (default: from xi and the thermal lengths)\n"
    "  --precision       fp64|fp32split         (default fp64)\n"
    "  --analysis        1: add ell, acf, q, psd beside each snapshot (default 0)\n"
    "  --field_file      float64 .npy field, shape (nx, ny), instead of the seeded one\n"
    "  --rows            R rows at unit spacing: --ny R --Ly R\n"
    "  --device          CUDA device            (default 0)\n";

struct Collect {
    std::vector<SnapshotOut> snaps;
    static void on(void *user, double t, const double *h, int n) {
        static_cast<Collect *>(user)->snaps.push_back(SnapshotOut{t, std::vector<double>(h, h + n)});
    }
};

int run(int argc, char **argv) {
    cli::Options a(argc, argv);
    if (a.help) {
        std::fputs(kUsage, stdout);
        return 0;
    }
    qew_dynamic_config cfg;
    qew_dynamic_config_default(&cfg);
    const std::string model = a.text("model", "arclength");
    cfg.model = cli::parse_model(model);
    cfg.amplitude = a.real("amplitude", 1.0);
    cfg.xi = a.real("xi", 0.1);
    cfg.pinning_length_over_xi = a.real("pinning_length", 0.1);
    cfg.driving_force = a.real("driving_force", 0.0);
    cfg.Lx = a.real("Lx", 2.0);
    cfg.Ly = a.real("Ly", 1.0);
    cfg.nx = a.integer("nx", 2048);
    cfg.ny = a.integer("ny", 1024);
    cli::apply_rows(a, cfg.ny, cfg.Ly);
    const std::vector<double> file_field = cli::field_from_file(a, cfg.nx, cfg.ny);
    cfg.seed = a.u64("seed", 1);
    cfg.tau = a.real("tau", 1.0);
    cfg.tl_start = a.real("tl_start", 0.01);
    cfg.tl_end = a.real("tl_end", 0.0001);
    cfg.total_time = a.real("total_time", 1000.0);
    const std::string fname = a.text("output", "dynamic_" + model + default_suffix());
    cfg.dt = a.real("dt", 0.0);
    cfg.precision = cli::parse_precision(a.text("precision", "fp64"));
    const bool analysis = a.integer("analysis", 0) != 0;
    const int device = a.integer("device", 0);
    a.finish();
    std::unique_ptr<Sink> sink = open_sink(fname);

    cli::Gpu gpu(device);
    const int store = QEW_STORE_FP64 | (cfg.precision == QEW_PREC_FP32_SPLIT ? QEW_STORE_FP32 : 0);
    gpu.field_for(file_field, cfg.nx, cfg.ny, cfg.Lx, cfg.Ly, cfg.amplitude, cfg.xi, cfg.seed,
                  store);
    Collect col;
    qew_dynamic_result res{};
    gpu.check(qew_dynamic_anneal(gpu.ctx, gpu.field, &cfg, &Collect::on, &col, &res),
              "dynamic_anneal");

    std::printf("dt=%.3g  total_time=%.3g  steps=%ld  line_tension=%.4g\n", res.dt, res.total_time,
                (long)(res.total_time / res.dt), res.line_tension);
    for (const SnapshotOut &s : col.snaps) std::printf("  saved t=%.6g\n", s.t);
    std::vector<LineStats> stats(col.snaps.size());
    if (analysis)
        for (size_t k = 0; k < col.snaps.size(); ++k) {
            stats[k] = cli::line_stats(gpu, col.snaps[k].h, cfg.Lx);
            col.snaps[k].stats = &stats[k];
        }
    write_dynamic(*sink, cfg, res.line_tension, col.snaps);
    sink->close();
    std::printf("wrote %s\n", fname.c_str());
    return 0;
}
}  // namespace

int main(int argc, char **argv) { return cli::guarded_main("qew_dynamic", kUsage, run, argc, argv); }
