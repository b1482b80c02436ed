// qew_cli_common.h -- what the three executables share: model and precision
// names, the GPU context and seeded field, and the exit-code convention
// (bad command line: message, usage, exit 2 -- as the reference's mains;
// a failure on the GPU: message, exit 1).
#pragma once

#include <cstdio>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

#include "qew_cli.h"
#include "qew_gpu.h"
#include "qew_io.h"
#include "qew_runs.h"

namespace qew {
namespace cli {

struct GpuError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline int parse_model(const std::string &name) {
    if (name == "linear") return QEW_MODEL_LINEAR;
    if (name == "arclength") return QEW_MODEL_ARCLENGTH;
    throw std::runtime_error("--model must be 'linear' or 'arclength', got '" + name + "'");
}

inline int parse_precision(const std::string &name) {
    if (name == "fp64") return QEW_PREC_FP64;
    if (name == "fp32split") return QEW_PREC_FP32_SPLIT;
    throw std::runtime_error("--precision must be 'fp64' or 'fp32split', got '" + name + "'");
}

// A context on one device and a seeded field; both released on scope exit.
class Gpu {
  public:
    explicit Gpu(int device) { check(qew_ctx_create(device, &ctx), "context"); }
    ~Gpu() {
        if (field) qew_field_destroy(field);
        if (ctx) qew_ctx_destroy(ctx);
    }
    // FilteredNoise(nx, ny, Lx, Ly, amplitude, xi, xi, seed) (the mains'
    // field, e.g. executables/qew_static/main.cpp:80-81).
    void seeded_field(int nx, int ny, double Lx, double Ly, double amplitude, double xi,
                      uint64_t seed, int store) {
        check(qew_field_create_seeded(ctx, nx, ny, Lx, Ly, amplitude, xi, xi, seed, store, &field),
              "field");
    }
    // FilteredNoise(field, nx, ny, Lx, Ly) (filtered_noise.h:186-189): a given
    // real-space field in the host layout [nx][ny].
    void host_field(const std::vector<double> &f, int nx, int ny, double Lx, double Ly, int store) {
        check(qew_field_create_from_host(ctx, f.data(), nx, ny, Lx, Ly, store, &field), "field");
    }
    // The executables' field: the file's when one was given, else the seeded one.
    void field_for(const std::vector<double> &file_field, int nx, int ny, double Lx, double Ly,
                   double amplitude, double xi, uint64_t seed, int store) {
        if (!file_field.empty())
            host_field(file_field, nx, ny, Lx, Ly, store);
        else
            seeded_field(nx, ny, Lx, Ly, amplitude, xi, seed, store);
    }
    void check(qew_status s, const char *what) {
        if (s != QEW_OK)
            throw GpuError(std::string(what) + ": " + qew_status_string(s) +
                           (ctx ? std::string(" (") + qew_last_error(ctx) + ")" : std::string()));
    }
    qew_ctx *ctx = nullptr;
    qew_field *field = nullptr;
};

// --rows R: R field rows at unit grid spacing (ny = R, Ly = R), the layout
// of the benchmark configurations. Not together with --ny or --Ly. Call it
// right after reading ny and Ly, before anything derived from them.
inline void apply_rows(Options &a, int &ny, double &Ly) {
    if (!a.has("rows")) return;
    if (a.has("ny") || a.has("Ly"))
        throw std::runtime_error("--rows sets --ny and --Ly; give either --rows or those");
    const int r = a.integer("rows", 0);
    if (r < 1) throw std::runtime_error("--rows must be positive");
    ny = r;
    Ly = (double)r;
}

// --field_file PATH: the real-space field as a float64 .npy array of shape
// (nx, ny), used in place of the seeded one (the reference's
// FilteredNoise(field, nx, ny, Lx, Ly)). Its shape sets nx and ny; --nx and
// --ny must match it when given. Returns an empty vector without the option.
inline std::vector<double> field_from_file(Options &a, int &nx, int &ny) {
    const std::string path = a.text("field_file", "");
    if (path.empty()) return {};
    int rows = 0, cols = 0;
    std::vector<double> f = read_npy_f64_2d(path, rows, cols);
    if ((a.has("nx") && rows != nx) || ((a.has("ny") || a.has("rows")) && cols != ny))
        throw std::runtime_error("--field_file '" + path + "' has shape (" + std::to_string(rows) +
                                 ", " + std::to_string(cols) + "), not the given --nx/--ny (" +
                                 std::to_string(nx) + ", " + std::to_string(ny) + ")");
    nx = rows;
    ny = cols;
    return f;
}

// ell, acf, q, psd of one host profile (qew_line_statistics_host).
inline LineStats line_stats(Gpu &gpu, const std::vector<double> &h, double L) {
    const int n = (int)h.size(), nh = n / 2 + 1;
    LineStats s;
    s.ell.resize(nh);
    s.acf.resize(nh);
    s.q.resize(nh);
    s.psd.resize(nh);
    gpu.check(qew_line_statistics_host(gpu.ctx, 1, h.data(), n, L, s.ell.data(), s.acf.data(),
                                       s.q.data(), s.psd.data()),
              "line_statistics");
    return s;
}

// main() body: run(argc, argv) with the exit-code convention.
template <class F>
int guarded_main(const char *prog, const char *usage, F run, int argc, char **argv) {
    try {
        return run(argc, argv);
    } catch (const GpuError &e) {
        std::fprintf(stderr, "%s: %s\n", prog, e.what());
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s: %s\n\n", prog, e.what());
        std::fputs(usage, stderr);
        return 2;
    }
}

}  // namespace cli
}  // namespace qew
