// Test probe for the executables' option reader and output writers
// (qew_gb300/csrc/cli/qew_cli.h, qew_io.h); host code only, no GPU.
//   QEW_PROBE=parse  reads the options of the reference's parser tests
//                    (tests/test_cli.cpp) and prints what it got;
//   QEW_PROBE=fmt    prints the key formatter's strings (test_executables.cpp:50-56);
//   QEW_PROBE=write  writes the three fixtures of test_executables.cpp:199-289
//                    as .npz files into the directory given as argv[1];
//   QEW_PROBE=npy    reads the float64 .npy array argv[1] (the --field_file
//                    reader) and prints its shape and a few values.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "qew_cli.h"
#include "qew_io.h"

using namespace qew;

static int parse(int argc, char **argv) {
    try {
        cli::Options a(argc, argv);
        std::printf("help=%d\n", a.help ? 1 : 0);
        std::printf("nx=%d\n", a.integer("nx", 4096));
        std::printf("ftol=%.17g\n", a.real("ftol", 1e-6));
        std::printf("seed=%llu\n", (unsigned long long)a.u64("seed", 1));
        std::printf("model=%s\n", a.text("model", "arclength").c_str());
        std::printf("driving_force=%.17g\n", a.real("driving_force", 0.0));
        const std::vector<double> l = a.real_list("pinning_lengths", {0.01, 0.1, 1.0});
        std::printf("pinning_lengths=");
        for (size_t k = 0; k < l.size(); ++k) std::printf("%s%.17g", k ? "," : "", l[k]);
        std::printf("\n");
        a.finish();
        return 0;
    } catch (const std::exception &e) {
        std::printf("error=%s\n", e.what());
        return 2;
    }
}

static int write(const std::string &dir) {
    {
        qew_static_config c{};
        c.Lx = 4.0;
        c.driving_force = 0.0;
        NpzSink s(dir + "/static.npz");
        write_static(s, c, {StaticOut{0.1, {1.0, 2.0, 3.0, 4.0}}});
        s.close();
    }
    {
        qew_dynamic_config c{};
        c.Lx = 2.0;
        c.driving_force = 0.0;
        c.pinning_length_over_xi = 0.1;
        NpzSink s(dir + "/dynamic.npz");
        write_dynamic(s, c, 2.0, {SnapshotOut{1.0, {5.0, 6.0}}});
        s.close();
    }
    {
        qew_depinning_config c{};
        c.Lx = 8.0;
        c.pinning_length_over_xi = 5.0;
        qew_depinning_result r{};
        r.f_c_upper_bound = 0.8;
        r.f_c = -1;
        NpzSink s(dir + "/depinning.npz");
        write_depinning(s, c, r, {DepinningOut{0.0, true, {0.5, 0.5, 0.5}},
                                  DepinningOut{0.8, false, {}}});
        s.close();
    }
    return 0;
}

int main(int argc, char **argv) {
    const char *mode = std::getenv("QEW_PROBE");
    const std::string m = mode ? mode : "parse";
    if (m == "fmt") {
        std::printf("%s|%s|%s|%s|%s\n", fmt("%.1g", 0.0).c_str(), fmt("%.3g", 0.1).c_str(),
                    fmt("%.3g", 100.0).c_str(), fmt("%.6g", 1.0).c_str(), fmt("%.4g", 0.8).c_str());
        return 0;
    }
    if (m == "write") return argc > 1 ? write(argv[1]) : 1;
    if (m == "npy") {
        if (argc < 2) return 1;
        try {
            int rows = 0, cols = 0;
            const std::vector<double> v = read_npy_f64_2d(argv[1], rows, cols);
            double sum = 0.0;
            for (double x : v) sum += x;
            std::printf("rows=%d\ncols=%d\nfirst=%.17g\nlast=%.17g\nsum=%.17g\n", rows, cols,
                        v.front(), v.back(), sum);
            return 0;
        } catch (const std::exception &e) {
            std::printf("error=%s\n", e.what());
            return 2;
        }
    }
    return parse(argc, argv);
}
