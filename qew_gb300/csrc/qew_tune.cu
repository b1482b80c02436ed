// qew_tune.cu -- the autotuner's per-process cache and its C entry points.
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "qew_tune.cuh"

namespace {

struct Entry {
    int choice;
    std::string detail;  // every candidate's time on the tuning call
};

std::mutex g_mu;
std::map<std::tuple<int, int, int>, Entry> g_cache;

const char *kKernelNames[kTuneKernels] = {"k_gradient_poly", "k_gradient_split_persist",
                                          "k_rk_resident", "k_langevin_run"};

}  // namespace

int qew_tune_class(long long points, int variant) {
    int b = 0;
    while (points > 1 && b < 62) {
        points >>= 1;
        ++b;
    }
    return 8 * b + (variant & 7);
}

int qew_tune_cached(int device, int kernel, int cls) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(std::make_tuple(device, kernel, cls));
    return it == g_cache.end() ? -1 : it->second.choice;
}

void qew_tune_remember(int device, int kernel, int cls, int choice, const std::string &detail) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[std::make_tuple(device, kernel, cls)] = Entry{choice, detail};
}

extern "C" {

qew_status qew_ctx_set_autotune(qew_ctx *ctx, int on) {
    if (!ctx) return QEW_ERR_INVALID;
    ctx->autotune = on ? 1 : 0;
    return QEW_OK;
}

qew_status qew_ctx_force_tune_candidate(qew_ctx *ctx, int kernel, int candidate) {
    if (!ctx || kernel < 0 || kernel >= kTuneKernels || candidate < -1)
        return qew_fail(ctx, QEW_ERR_INVALID, "force_tune_candidate: bad arguments");
    ctx->tune_force[kernel] = candidate;
    return QEW_OK;
}

int qew_tune_report(char *buf, int size) {
    std::string out;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        for (const auto &kv : g_cache) {
            char head[160];
            snprintf(head, sizeof(head), "device %d %s class %d: candidate %d [",
                     std::get<0>(kv.first), kKernelNames[std::get<1>(kv.first)],
                     std::get<2>(kv.first), kv.second.choice);
            out += head;
            out += kv.second.detail;
            out += "]\n";
        }
    }
    if (buf && size > 0) {
        const size_t k = out.size() < (size_t)size - 1 ? out.size() : (size_t)size - 1;
        memcpy(buf, out.data(), k);
        buf[k] = '\0';
    }
    return (int)out.size();
}

}  // extern "C"
