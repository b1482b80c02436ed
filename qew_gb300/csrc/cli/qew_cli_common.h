// qew_cli_common.h -- what the three executables share: model and precision
// names, the GPU context and seeded field, and the exit-code convention
// (bad command line: message, usage, exit 2 -- as the reference's mains;
// a failure on the GPU: message, exit 1).
#pragma once

#include <cstdio>
#include <exception>
#include <stdexcept>
#include <string>

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
    void check(qew_status s, const char *what) {
        if (s != QEW_OK)
            throw GpuError(std::string(what) + ": " + qew_status_string(s) +
                           (ctx ? std::string(" (") + qew_last_error(ctx) + ")" : std::string()));
    }
    qew_ctx *ctx = nullptr;
    qew_field *field = nullptr;
};

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
