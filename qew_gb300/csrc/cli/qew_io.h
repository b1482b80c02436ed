// qew_io.h -- output of the three simulation executables (and the .npy
// reader of their --field_file input).
//
// The dataset KEYS are the reference's contract with its analysis scripts
// (qew_io.h:22-63, qew_format.h:13-17, pinned by test_executables.cpp:50-56
// and 199-289): the same printf specs build the same strings here. Where the
// values go is a Sink: an uncompressed NumPy .npz archive (always built; its
// member names are exactly the keys, so np.load(...)[key] reads them) and,
// when compiled with QEW_WITH_HDF5 and the HDF5 C library, an HDF5 file with
// the same paths (groups created on the way).
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "qew_runs.h"

#ifdef QEW_WITH_HDF5
#include <hdf5.h>
#endif

namespace qew {

// A float64 2-D array from a .npy file (format versions 1-3, little-endian
// '<f8', C order), e.g. the real-space field of --field_file: shape (nx, ny),
// x slow and y fast, the reference's host layout (filtered_noise.h:208).
// Anything else (another dtype, Fortran order, another rank, a short file)
// is an error.
inline std::vector<double> read_npy_f64_2d(const std::string &path, int &rows, int &cols) {
    const uint16_t one = 1;
    unsigned char lsb;
    std::memcpy(&lsb, &one, 1);
    if (lsb != 1) throw std::runtime_error("reading .npy needs a little-endian host");
    std::unique_ptr<std::FILE, int (*)(std::FILE *)> f(std::fopen(path.c_str(), "rb"), &std::fclose);
    if (!f) throw std::runtime_error("cannot open '" + path + "'");
    const std::string what = "'" + path + "': ";
    unsigned char pre[8];
    if (std::fread(pre, 1, 8, f.get()) != 8 || std::memcmp(pre, "\x93NUMPY", 6) != 0)
        throw std::runtime_error(what + "not a .npy file");
    size_t hlen = 0;
    if (pre[6] == 1) {
        unsigned char b[2];
        if (std::fread(b, 1, 2, f.get()) != 2) throw std::runtime_error(what + "short header");
        hlen = (size_t)b[0] | (size_t)b[1] << 8;
    } else if (pre[6] == 2 || pre[6] == 3) {
        unsigned char b[4];
        if (std::fread(b, 1, 4, f.get()) != 4) throw std::runtime_error(what + "short header");
        hlen = (size_t)b[0] | (size_t)b[1] << 8 | (size_t)b[2] << 16 | (size_t)b[3] << 24;
    } else {
        throw std::runtime_error(what + "unsupported .npy version");
    }
    if (hlen == 0 || hlen > (1u << 20)) throw std::runtime_error(what + "bad header length");
    std::string hdr(hlen, '\0');
    if (std::fread(&hdr[0], 1, hlen, f.get()) != hlen) throw std::runtime_error(what + "short header");
    auto value_of = [&](const char *key) {  // text after 'key': up to the next ',' or '}' at depth 0
        const std::string k = std::string("'") + key + "'";
        size_t at = hdr.find(k);
        if (at == std::string::npos) throw std::runtime_error(what + "header lacks " + k);
        at = hdr.find(':', at + k.size());
        if (at == std::string::npos) throw std::runtime_error(what + "bad header");
        size_t end = at + 1;
        int depth = 0;
        for (; end < hdr.size(); ++end) {
            const char c = hdr[end];
            if (c == '(') ++depth;
            if (c == ')') --depth;
            if (depth == 0 && (c == ',' || c == '}')) break;
        }
        std::string v = hdr.substr(at + 1, end - at - 1);
        const size_t b = v.find_first_not_of(" "), e = v.find_last_not_of(" ");
        return b == std::string::npos ? std::string() : v.substr(b, e - b + 1);
    };
    if (value_of("descr") != "'<f8'") throw std::runtime_error(what + "dtype must be float64 ('<f8')");
    if (value_of("fortran_order") != "False") throw std::runtime_error(what + "must be C order");
    const std::string shape = value_of("shape");
    std::vector<long long> d;  // the tuple's items: "(a, b)", spaces and a trailing comma allowed
    if (shape.size() < 2 || shape.front() != '(' || shape.back() != ')')
        throw std::runtime_error(what + "bad shape " + shape);
    size_t pos = 1;
    while (pos < shape.size() - 1) {
        size_t comma = shape.find(',', pos);
        if (comma == std::string::npos || comma > shape.size() - 1) comma = shape.size() - 1;
        std::string item = shape.substr(pos, comma - pos);
        item.erase(0, item.find_first_not_of(' '));
        item.erase(item.find_last_not_of(' ') + 1);
        if (!item.empty()) {
            char *end = nullptr;
            const long long v = std::strtoll(item.c_str(), &end, 10);
            if (*end != '\0') throw std::runtime_error(what + "bad shape " + shape);
            d.push_back(v);
        }
        pos = comma + 1;
    }
    if (d.size() != 2) throw std::runtime_error(what + "must be a 2-D array, shape " + shape);
    if (d[0] < 1 || d[1] < 1 || d[0] > INT32_MAX || d[1] > INT32_MAX)
        throw std::runtime_error(what + "bad shape " + shape);
    const size_t count = (size_t)d[0] * (size_t)d[1];
    std::vector<double> out(count);
    if (std::fread(out.data(), sizeof(double), count, f.get()) != count)
        throw std::runtime_error(what + "fewer values than its shape");
    rows = (int)d[0];
    cols = (int)d[1];
    return out;
}

// printf into a std::string (qew_format.h:13-17).
inline std::string fmt(const char *spec, double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), spec, v);
    return std::string(buf);
}

class Sink {
  public:
    virtual ~Sink() = default;
    virtual void scalar(const std::string &key, double v) = 0;
    virtual void vector(const std::string &key, const std::vector<double> &v) = 0;
    virtual void close() {}
};

// ---------------------------------------------------------------- .npz
// A stored (uncompressed) ZIP archive of .npy members, little-endian
// throughout, written in one pass at close().
class NpzSink : public Sink {
  public:
    explicit NpzSink(std::string fname) : fname_(std::move(fname)) {}
    ~NpzSink() override {
        try {
            close();
        } catch (...) {
        }
    }
    void scalar(const std::string &key, double v) override { add(key, {v}, true); }
    void vector(const std::string &key, const std::vector<double> &v) override { add(key, v, false); }
    void close() override {
        if (closed_) return;
        closed_ = true;
        std::FILE *fp = std::fopen(fname_.c_str(), "wb");
        if (!fp) throw std::runtime_error("cannot open '" + fname_ + "' for writing");
        std::vector<uint8_t> central;
        uint64_t off = 0;
        for (const Member &m : members_) {
            const uint32_t crc = crc32(m.bytes);
            const uint64_t size = m.bytes.size();
            if (off > 0xffffffffULL || size > 0xffffffffULL)
                throw std::runtime_error("npz output above 4 GiB");
            std::vector<uint8_t> lh;
            put32(lh, 0x04034b50u);
            put16(lh, 20);  // version needed
            put16(lh, 0);   // flags
            put16(lh, 0);   // stored
            put16(lh, 0);   // time
            put16(lh, 0x21);  // date 1980-01-01
            put32(lh, crc);
            put32(lh, (uint32_t)size);
            put32(lh, (uint32_t)size);
            put16(lh, (uint16_t)m.name.size());
            put16(lh, 0);
            lh.insert(lh.end(), m.name.begin(), m.name.end());
            write(fp, lh);
            write(fp, m.bytes);
            put32(central, 0x02014b50u);
            put16(central, 20);  // made by
            put16(central, 20);  // needed
            put16(central, 0);
            put16(central, 0);
            put16(central, 0);
            put16(central, 0x21);
            put32(central, crc);
            put32(central, (uint32_t)size);
            put32(central, (uint32_t)size);
            put16(central, (uint16_t)m.name.size());
            put16(central, 0);  // extra
            put16(central, 0);  // comment
            put16(central, 0);  // disk
            put16(central, 0);  // internal attributes
            put32(central, 0);  // external attributes
            put32(central, (uint32_t)off);
            central.insert(central.end(), m.name.begin(), m.name.end());
            off += lh.size() + size;
        }
        if (off > 0xffffffffULL) throw std::runtime_error("npz output above 4 GiB");
        std::vector<uint8_t> end;
        put32(end, 0x06054b50u);
        put16(end, 0);
        put16(end, 0);
        put16(end, (uint16_t)members_.size());
        put16(end, (uint16_t)members_.size());
        put32(end, (uint32_t)central.size());
        put32(end, (uint32_t)off);
        put16(end, 0);
        write(fp, central);
        write(fp, end);
        if (std::fclose(fp) != 0) throw std::runtime_error("error writing '" + fname_ + "'");
    }

  private:
    struct Member {
        std::string name;
        std::vector<uint8_t> bytes;
    };
    static void put16(std::vector<uint8_t> &b, uint16_t v) {
        b.push_back((uint8_t)(v & 0xff));
        b.push_back((uint8_t)(v >> 8));
    }
    static void put32(std::vector<uint8_t> &b, uint32_t v) {
        for (int k = 0; k < 4; ++k) b.push_back((uint8_t)((v >> (8 * k)) & 0xff));
    }
    static void write(std::FILE *fp, const std::vector<uint8_t> &b) {
        if (!b.empty() && std::fwrite(b.data(), 1, b.size(), fp) != b.size())
            throw std::runtime_error("short write");
    }
    // CRC-32 (ISO 3309 / ITU-T V.42, reflected polynomial 0xEDB88320).
    static uint32_t crc32(const std::vector<uint8_t> &b) {
        static uint32_t table[256];
        static bool init = false;
        if (!init) {
            for (uint32_t i = 0; i < 256; ++i) {
                uint32_t c = i;
                for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
                table[i] = c;
            }
            init = true;
        }
        uint32_t c = 0xffffffffu;
        for (uint8_t x : b) c = table[(c ^ x) & 0xff] ^ (c >> 8);
        return c ^ 0xffffffffu;
    }
    // NPY format 1.0: magic, version, header length, a Python-literal dict
    // padded with spaces to a multiple of 64 bytes, then the raw '<f8' data.
    void add(const std::string &key, const std::vector<double> &v, bool is_scalar) {
        for (const Member &m : members_)
            if (m.name == key + ".npy") throw std::runtime_error("duplicate key '" + key + "'");
        std::string dict = "{'descr': '<f8', 'fortran_order': False, 'shape': (";
        if (!is_scalar) dict += std::to_string(v.size()) + ",";
        dict += "), }";
        size_t total = 10 + dict.size() + 1;
        const size_t pad = (64 - total % 64) % 64;
        dict.append(pad, ' ');
        dict += '\n';
        Member m;
        m.name = key + ".npy";
        const char magic[] = "\x93NUMPY";
        m.bytes.insert(m.bytes.end(), magic, magic + 6);
        m.bytes.push_back(1);
        m.bytes.push_back(0);
        put16(m.bytes, (uint16_t)dict.size());
        m.bytes.insert(m.bytes.end(), dict.begin(), dict.end());
        for (double x : v) {
            uint64_t u;
            std::memcpy(&u, &x, 8);
            for (int k = 0; k < 8; ++k) m.bytes.push_back((uint8_t)((u >> (8 * k)) & 0xff));
        }
        members_.push_back(std::move(m));
    }
    std::string fname_;
    std::vector<Member> members_;
    bool closed_ = false;
};

#ifdef QEW_WITH_HDF5
// ----------------------------------------------------------------- HDF5
class Hdf5Sink : public Sink {
  public:
    explicit Hdf5Sink(const std::string &fname) {
        file_ = H5Fcreate(fname.c_str(), H5F_ACC_TRUNC, H5P_DEFAULT, H5P_DEFAULT);
        if (file_ < 0) throw std::runtime_error("cannot create '" + fname + "'");
        lcpl_ = H5Pcreate(H5P_LINK_CREATE);
        H5Pset_create_intermediate_group(lcpl_, 1);
    }
    ~Hdf5Sink() override { close(); }
    void scalar(const std::string &key, double v) override { put(key, H5Screate(H5S_SCALAR), &v); }
    void vector(const std::string &key, const std::vector<double> &v) override {
        const hsize_t d = v.size();
        put(key, H5Screate_simple(1, &d, nullptr), v.data());
    }
    void close() override {
        if (file_ >= 0) {
            H5Pclose(lcpl_);
            H5Fclose(file_);
            file_ = -1;
        }
    }

  private:
    void put(const std::string &key, hid_t space, const double *data) {
        const hid_t ds = H5Dcreate2(file_, key.c_str(), H5T_NATIVE_DOUBLE, space, lcpl_, H5P_DEFAULT,
                                    H5P_DEFAULT);
        if (ds < 0) {
            H5Sclose(space);
            throw std::runtime_error("cannot create dataset '" + key + "'");
        }
        const herr_t e = H5Dwrite(ds, H5T_NATIVE_DOUBLE, H5S_ALL, H5S_ALL, H5P_DEFAULT, data);
        H5Dclose(ds);
        H5Sclose(space);
        if (e < 0) throw std::runtime_error("cannot write dataset '" + key + "'");
    }
    hid_t file_ = -1, lcpl_ = -1;
};
#endif

inline bool ends_with(const std::string &s, const std::string &suf) {
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

// The default output suffix: .h5 where HDF5 is compiled in, else .npz.
inline const char *default_suffix() {
#ifdef QEW_WITH_HDF5
    return ".h5";
#else
    return ".npz";
#endif
}

// A sink for `fname`, chosen by its suffix.
inline std::unique_ptr<Sink> open_sink(const std::string &fname) {
    if (ends_with(fname, ".npz")) return std::unique_ptr<Sink>(new NpzSink(fname));
#ifdef QEW_WITH_HDF5
    return std::unique_ptr<Sink>(new Hdf5Sink(fname));
#else
    throw std::runtime_error("compiled without the HDF5 writer: give --output a .npz name (got '" +
                             fname + "')");
#endif
}

// ------------------------------------------------------------ the writers
// Roughness statistics written beside a profile (the datasets the reference's
// post-processing adds to every ".../h" group: ell, acf, q, psd;
// tools/postprocess_static.py:38-46), when the executable is asked for them.
struct LineStats {
    std::vector<double> ell, acf, q, psd;
};

inline void write_line_stats(Sink &s, const std::string &prefix, const LineStats *st) {
    if (!st) return;
    s.vector(prefix + "/ell", st->ell);
    s.vector(prefix + "/acf", st->acf);
    s.vector(prefix + "/q", st->q);
    s.vector(prefix + "/psd", st->psd);
}

struct StaticOut {
    double pinning_length_over_xi;
    std::vector<double> h;
    const LineStats *stats = nullptr;
};

// write_static, qew_io.h:24-34.
inline void write_static(Sink &s, const qew_static_config &c, const std::vector<StaticOut> &profiles) {
    s.scalar("physical_size", c.Lx);
    for (const StaticOut &p : profiles) {
        const std::string prefix = "driving_force=" + fmt("%.1g", c.driving_force) +
                                   "/pinning_length=" + fmt("%.3g", p.pinning_length_over_xi);
        s.scalar(prefix + "/pinning_length", p.pinning_length_over_xi);
        s.vector(prefix + "/h", p.h);
        write_line_stats(s, prefix, p.stats);
    }
}

struct SnapshotOut {
    double t;
    std::vector<double> h;
    const LineStats *stats = nullptr;
};

// write_dynamic, qew_io.h:36-48.
inline void write_dynamic(Sink &s, const qew_dynamic_config &c, double line_tension,
                          const std::vector<SnapshotOut> &snaps) {
    s.scalar("physical_size", c.Lx);
    for (const SnapshotOut &sn : snaps) {
        const std::string prefix = "timestep=" + fmt("%.6g", sn.t) + "/driving_force=" +
                                   fmt("%.1g", c.driving_force) + "/line_tension=" +
                                   fmt("%.3g", line_tension);
        s.scalar(prefix + "/pinning_length", c.pinning_length_over_xi);
        s.vector(prefix + "/h", sn.h);
        write_line_stats(s, prefix, sn.stats);
    }
}

struct DepinningOut {
    double f;
    bool blocked;
    std::vector<double> h;  // blocked steps only
    const LineStats *stats = nullptr;
};

// write_depinning, qew_io.h:50-63; f_c (bisection) is an added key, written
// only when the bisection ran.
inline void write_depinning(Sink &s, const qew_depinning_config &c, const qew_depinning_result &r,
                            const std::vector<DepinningOut> &steps) {
    s.scalar("physical_size", c.Lx);
    for (const DepinningOut &st : steps) {
        if (!st.blocked) continue;
        const std::string prefix = "driving_force=" + fmt("%.4g", st.f);
        s.vector(prefix + "/h", st.h);
        s.scalar(prefix + "/pinning_length", c.pinning_length_over_xi);
        write_line_stats(s, prefix, st.stats);
    }
    if (r.f_c_upper_bound >= 0) s.scalar("f_c_upper_bound", r.f_c_upper_bound);
    if (r.f_c >= 0) s.scalar("f_c", r.f_c);
}

}  // namespace qew
