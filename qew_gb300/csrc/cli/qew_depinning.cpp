// qew_depinning -- Rosso-Krauth force ramp toward f_c, the executable of the
// reference's depinning run (executables/qew_depinning/main.cpp) with the
// same options, defaults (RK knobs derived from Ly/ny), console lines and
// output keys, on the GPU. Added options: --bisect_rtol (bisect f_c after
// the ramp; adds the key f_c), --precision fp64|fp32split, --analysis 1 (ell,
// acf, q, psd beside each blocked profile), --field_file (a given field),
// --rows (unit-spacing rows), --device.
#include <cstdio>
#include <string>
#include <vector>

#include "qew_cli_common.h"

using namespace qew;

namespace {
const char *kUsage =
    "qew_depinning -- Rosso-Krauth force ramp toward the threshold f_c (GPU).\n"
    "All options take a value.\n\n"
    "  --model           linear|arclength      (default arclength)\n"
    "  --amplitude       disorder amplitude U0  (default 1)\n"
    "  --xi              correlation length     (default 0.1)\n"
    "  --pinning_length  lambda_p/xi (stiff)    (default 5)\n"
    "  --Lx --Ly         system size            (default 8, 1)\n"
    "  --nx --ny         resolution             (default 1024, 256)\n"
    "  --f_step          force ramp increment   (default 1)\n"
    "  --f_max           force ramp cap         (default 40)\n"
    "  --seed            noise RNG seed         (default 1)\n"
    "  --output          output file            (default depinning_<model>.npz, .h5 with HDF5)\n"
    "  RK solver knobs (defaults derived from Ly/ny):\n"
    "  --dstep --max_advance --runaway --root_tol --sweep_tol --max_sweeps\n"
    "  --bisect_rtol     bisect f_c to this relative width after the ramp (default 0: off)\n"
    "  --precision       fp64|fp32split         (default fp64)\n"
    "  --analysis        1: add ell, acf, q, psd beside each blocked profile (default 0)\n"
    "  --field_file      float64 .npy field, shape (nx, ny), instead of the seeded one\n"
    "  --rows            R rows at unit spacing: --ny R --Ly R\n"
    "  --device          CUDA device            (default 0)\n";

struct Collect {
    std::vector<DepinningOut> steps;
    std::vector<qew_depinning_step> raw;
    static void on(void *user, const qew_depinning_step *st, const double *h, int n) {
        Collect *c = static_cast<Collect *>(user);
        c->raw.push_back(*st);
        c->steps.push_back(DepinningOut{st->f, st->result.blocked != 0,
                                        h ? std::vector<double>(h, h + n) : std::vector<double>()});
    }
};

int run(int argc, char **argv) {
    cli::Options a(argc, argv);
    if (a.help) {
        std::fputs(kUsage, stdout);
        return 0;
    }
    qew_depinning_config cfg;
    qew_depinning_config_default(&cfg);
    const std::string model = a.text("model", "arclength");
    cfg.model = cli::parse_model(model);
    cfg.amplitude = a.real("amplitude", 1.0);
    cfg.xi = a.real("xi", 0.1);
    cfg.pinning_length_over_xi = a.real("pinning_length", 5.0);
    cfg.Lx = a.real("Lx", 8.0);
    cfg.Ly = a.real("Ly", 1.0);
    cfg.nx = a.integer("nx", 1024);
    cfg.ny = a.integer("ny", 256);
    cli::apply_rows(a, cfg.ny, cfg.Ly);
    const std::vector<double> file_field = cli::field_from_file(a, cfg.nx, cfg.ny);
    cfg.f_step = a.real("f_step", 1.0);
    cfg.f_max = a.real("f_max", 40.0);
    cfg.rp.dstep = a.real("dstep", 0.5 * (cfg.Ly / cfg.ny));
    cfg.rp.max_advance = a.real("max_advance", cfg.Ly);
    cfg.rp.runaway = a.real("runaway", 2.0 * cfg.Ly);
    cfg.rp.root_tol = a.real("root_tol", 1e-10);
    cfg.rp.sweep_tol = a.real("sweep_tol", 1e-8);
    cfg.rp.max_sweeps = a.integer("max_sweeps", 200000);
    const uint64_t seed = a.u64("seed", 1);
    const std::string fname = a.text("output", "depinning_" + model + default_suffix());
    cfg.bisect_rtol = a.real("bisect_rtol", 0.0);
    cfg.precision = cli::parse_precision(a.text("precision", "fp64"));
    const bool analysis = a.integer("analysis", 0) != 0;
    const int device = a.integer("device", 0);
    a.finish();
    std::unique_ptr<Sink> sink = open_sink(fname);

    cli::Gpu gpu(device);
    const int store = QEW_STORE_FP64 | (cfg.precision == QEW_PREC_FP32_SPLIT ? QEW_STORE_FP32 : 0);
    gpu.field_for(file_field, cfg.nx, cfg.ny, cfg.Lx, cfg.Ly, cfg.amplitude, cfg.xi, seed, store);
    Collect col;
    qew_depinning_result res{};
    gpu.check(qew_depinning_ramp(gpu.ctx, gpu.field, &cfg, &Collect::on, &col, &res),
              "depinning_ramp");

    std::printf("model=%s  lambda_p/xi=%.3g  line_tension=%.4g\n", model.c_str(),
                cfg.pinning_length_over_xi, res.line_tension);
    for (const qew_depinning_step &st : col.raw)
        std::printf("f=%7.3f  sweeps=%-7d mean_h=%8.4f  %s\n", st.f, st.result.sweeps,
                    st.result.mean_h,
                    st.result.blocked ? "blocked" : (st.result.runaway ? "DEPINNED" : "timeout"));
    if (res.f_c_upper_bound >= 0)
        std::printf("Line depinned near f=%.3f; stopping ramp.\n", res.f_c_upper_bound);
    if (res.f_c >= 0)
        std::printf("f_c=%.10g  bracket [%.10g, %.10g]  %d bisection blocks\n", res.f_c,
                    res.f_c_lo, res.f_c_hi, res.bisect_blocks);
    std::vector<LineStats> stats(col.steps.size());
    if (analysis)
        for (size_t k = 0; k < col.steps.size(); ++k)
            if (col.steps[k].blocked) {
                stats[k] = cli::line_stats(gpu, col.steps[k].h, cfg.Lx);
                col.steps[k].stats = &stats[k];
            }
    write_depinning(*sink, cfg, res, col.steps);
    sink->close();
    std::printf("wrote %s\n", fname.c_str());
    return 0;
}
}  // namespace

int main(int argc, char **argv) {
    return cli::guarded_main("qew_depinning", kUsage, run, argc, argv);
}
