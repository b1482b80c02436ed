// qew_cli.h -- the `--key value` / `--key=value` option reader of the three
// simulation executables, with the reference's rules (executables/cli.h,
// pinned by tests/test_cli.cpp):
//   * every option takes a value; --help and -h are the only flags;
//   * the value is the next token even when it starts with '-' (negative
//     numbers), unless the option is written --key=value;
//   * a token that does not start with "--" is an error, as is a trailing
//     option without a value or an empty option name;
//   * defaults are given where an option is read; numbers must parse in
//     full; comma lists skip empty items and may not be empty;
//   * after reading, finish() rejects options that nothing read.
// Dependency-free (standard library only), so the parser tests build it
// alone.
#pragma once

#include <cstdint>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace qew {
namespace cli {

class Options {
  public:
    Options(int argc, char **argv) {
        int i = 1;
        while (i < argc) {
            const std::string tok = argv[i++];
            if (tok == "--help" || tok == "-h") {
                help = true;
                continue;
            }
            if (tok.size() < 2 || tok[0] != '-' || tok[1] != '-')
                throw std::runtime_error("unexpected argument '" + tok +
                                         "' (options start with --)");
            const std::string body = tok.substr(2);
            const size_t eq = body.find('=');
            std::string key, val;
            if (eq != std::string::npos) {
                key = body.substr(0, eq);
                val = body.substr(eq + 1);
            } else {
                if (i >= argc) throw std::runtime_error("option --" + body + " needs a value");
                key = body;
                val = argv[i++];
            }
            if (key.empty()) throw std::runtime_error("empty option name in '" + tok + "'");
            given_[key] = val;
        }
    }

    bool help = false;

    bool has(const std::string &k) const { return given_.count(k) > 0; }

    std::string text(const std::string &k, const std::string &def) {
        const std::string *v = take(k);
        return v ? *v : def;
    }
    double real(const std::string &k, double def) {
        const std::string *v = take(k);
        return v ? number<double>(k, *v) : def;
    }
    int integer(const std::string &k, int def) {
        const std::string *v = take(k);
        return v ? number<int>(k, *v) : def;
    }
    uint64_t u64(const std::string &k, uint64_t def) {
        const std::string *v = take(k);
        return v ? number<uint64_t>(k, *v) : def;
    }
    std::vector<double> real_list(const std::string &k, const std::vector<double> &def) {
        const std::string *v = take(k);
        if (!v) return def;
        std::vector<double> out;
        size_t start = 0;
        while (start <= v->size()) {
            size_t comma = v->find(',', start);
            if (comma == std::string::npos) comma = v->size();
            const std::string item = v->substr(start, comma - start);
            if (!item.empty()) out.push_back(number<double>(k, item));
            start = comma + 1;
        }
        if (out.empty()) throw std::runtime_error("option --" + k + ": empty list '" + *v + "'");
        return out;
    }

    // Every option given must have been read.
    void finish() const {
        std::string bad;
        for (const auto &kv : given_) {
            if (read_.count(kv.first)) continue;
            if (!bad.empty()) bad += ", ";
            bad += "--" + kv.first;
        }
        if (!bad.empty()) throw std::runtime_error("unknown option(s): " + bad);
    }

  private:
    const std::string *take(const std::string &k) {
        const auto it = given_.find(k);
        if (it == given_.end()) return nullptr;
        read_.insert(k);
        return &it->second;
    }
    template <class T>
    static T number(const std::string &k, const std::string &text) {
        std::istringstream in(text);
        T v{};
        in >> v;
        if (in.fail() || in.peek() != std::char_traits<char>::eof())
            throw std::runtime_error("option --" + k + ": cannot parse '" + text + "' as a number");
        return v;
    }
    std::map<std::string, std::string> given_;
    std::set<std::string> read_;
};

}  // namespace cli
}  // namespace qew
