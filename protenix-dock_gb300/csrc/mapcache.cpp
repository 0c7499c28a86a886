// Codec of the reference's map cache files (see mapcache.h), restating the published
// Boost.Serialization archive layouts that receptor_cache::save writes (grid.cpp:309-345,
// 394-406), with this library's own readers and writers.
//
// Binary archive of std::vector<val_and_grad> (little-endian, as both hosts are):
//   u64 22, "serialization::archive"      signature (std::string: size_t length + bytes)
//   u16 library version                   (library_version_type)
//   u8 4, u8 8, u8 4, u8 8                sizeof int, long, float, double
//   i32 1                                 byte-order check
//   u8 tracking, u32 class version        the vector's class preamble (first object of
//                                         its type; binary archives omit the class id)
//   u64 count                             collection_size_type
//   u32 item version                      item_version_type
//   per point: E, dE/dx, dE/dy, dE/dz as param_t, the first point carrying the
//   preambles of val_and_grad (before E) and atom_position (before the gradient).
// Text archive meta.dat: space-separated tokens "22 serialization::archive <lib>", the
// format version, the C arrays init_xyz and npoints as "3 a b c", the spacing in
// scientific notation with max_digits10 digits, then the unordered_set of excluded atom
// indices: its preamble "0 0", count, bucket count, item version, the items; a newline
// ends the archive.
#include "mapcache.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <stdexcept>

namespace pxd {
namespace mapcache {

namespace {

const char kSignature[] = "serialization::archive";
constexpr size_t kSigLen = sizeof(kSignature) - 1;  // 22

// header + vector preamble + count + item version
constexpr size_t kHeadBytes = 8 + kSigLen + 2 + 4 + 4;
constexpr size_t kPrologueBytes = kHeadBytes + 1 + 4 + 8 + 4;
// the two element preambles carried by the first point
constexpr size_t kFirstPointExtra = 2 * (1 + 4);

struct Writer {
    std::vector<uint8_t> out;
    template <class T>
    void put(T v) {
        uint8_t b[sizeof(T)];
        std::memcpy(b, &v, sizeof(T));
        out.insert(out.end(), b, b + sizeof(T));
    }
    void put_value(double v, int value_bytes) {
        if (value_bytes == 8)
            put<double>(v);
        else
            put<float>(static_cast<float>(v));
    }
};

struct Reader {
    const uint8_t* p;
    size_t n, at = 0;
    template <class T>
    T get() {
        if (n - at < sizeof(T)) throw std::runtime_error("map archive is truncated");
        T v;
        std::memcpy(&v, p + at, sizeof(T));
        at += sizeof(T);
        return v;
    }
};

void check_preamble(Reader& r) {
    const uint8_t tracking = r.get<uint8_t>();
    const uint32_t version = r.get<uint32_t>();
    if (tracking > 1 || version != 0) throw std::runtime_error("map archive: unexpected class preamble");
}

}  // namespace

std::vector<uint8_t> encode_bdg(const double* records, size_t n_points, int value_bytes) {
    if (value_bytes != 8 && value_bytes != 4) throw std::runtime_error("map archive values are 8 or 4 bytes");
    Writer w;
    w.out.reserve(kPrologueBytes + kFirstPointExtra + n_points * 4 * value_bytes);
    w.put<uint64_t>(kSigLen);
    w.out.insert(w.out.end(), kSignature, kSignature + kSigLen);
    w.put<uint16_t>(kWriteLibraryVersion);
    w.put<uint8_t>(4);
    w.put<uint8_t>(8);
    w.put<uint8_t>(4);
    w.put<uint8_t>(8);
    w.put<int32_t>(1);
    w.put<uint8_t>(0);   // std::vector: not tracked
    w.put<uint32_t>(0);  // class version
    w.put<uint64_t>(n_points);
    w.put<uint32_t>(0);  // item version of val_and_grad
    for (size_t i = 0; i < n_points; ++i) {
        const double* r = records + 4 * i;
        if (i == 0) {
            w.put<uint8_t>(0);
            w.put<uint32_t>(0);
        }
        w.put_value(r[0], value_bytes);
        if (i == 0) {
            w.put<uint8_t>(0);
            w.put<uint32_t>(0);
        }
        w.put_value(r[1], value_bytes);
        w.put_value(r[2], value_bytes);
        w.put_value(r[3], value_bytes);
    }
    return w.out;
}

std::vector<double> decode_bdg(const uint8_t* data, size_t size, int* value_bytes) {
    Reader r{data, size};
    if (r.get<uint64_t>() != kSigLen || size < r.at + kSigLen || std::memcmp(data + r.at, kSignature, kSigLen) != 0)
        throw std::runtime_error("not a Boost binary archive (signature)");
    r.at += kSigLen;
    const uint16_t lib = r.get<uint16_t>();
    if (lib < 8) throw std::runtime_error("Boost archive library version " + std::to_string(lib) + " is older than 8");
    const uint8_t s_int = r.get<uint8_t>(), s_long = r.get<uint8_t>(), s_float = r.get<uint8_t>(),
                  s_double = r.get<uint8_t>();
    if (s_int != 4 || s_long != 8 || s_float != 4 || s_double != 8)
        throw std::runtime_error("map archive written on a host with other type sizes");
    if (r.get<int32_t>() != 1) throw std::runtime_error("map archive written on a big-endian host");
    check_preamble(r);
    const uint64_t count = r.get<uint64_t>();
    r.get<uint32_t>();  // item version
    const size_t rest = size - r.at;
    int vb = 0;
    if (count == 0) {
        if (rest != 0) throw std::runtime_error("map archive: bytes after an empty map");
        vb = 8;
    } else if (rest >= kFirstPointExtra && count <= (rest - kFirstPointExtra) / 16) {
        const size_t body = rest - kFirstPointExtra;
        if (body == count * 32)
            vb = 8;
        else if (body == count * 16)
            vb = 4;
    }
    if (!vb) throw std::runtime_error("map archive: length does not match its point count");
    std::vector<double> rec(count * 4);
    for (uint64_t i = 0; i < count; ++i) {
        double* o = rec.data() + 4 * i;
        if (i == 0) check_preamble(r);
        o[0] = vb == 8 ? r.get<double>() : static_cast<double>(r.get<float>());
        if (i == 0) check_preamble(r);
        for (int c = 1; c < 4; ++c) o[c] = vb == 8 ? r.get<double>() : static_cast<double>(r.get<float>());
    }
    if (value_bytes) *value_bytes = vb;
    return rec;
}

namespace {

std::string sci(double v) {
    // std::scientific with max_digits10 digits after the point, as Boost's text archive
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.*e", std::numeric_limits<double>::max_digits10, v);
    return buf;
}

// the smallest prime >= n (at least 1): a bucket count for the unordered_set record
uint64_t bucket_count_for(uint64_t n) {
    auto prime = [](uint64_t v) {
        if (v < 2) return false;
        for (uint64_t d = 2; d * d <= v; ++d)
            if (v % d == 0) return false;
        return true;
    };
    uint64_t v = n < 2 ? 1 : n;
    if (v == 1) return 1;
    while (!prime(v)) ++v;
    return v;
}

struct Tokens {
    std::istringstream in;
    explicit Tokens(const std::string& s) : in(s) {}
    std::string next() {
        std::string t;
        if (!(in >> t)) throw std::runtime_error("meta.dat is truncated");
        return t;
    }
    uint64_t u64() {
        const std::string t = next();
        char* end = nullptr;
        const unsigned long long v = std::strtoull(t.c_str(), &end, 10);
        if (t.empty() || *end || t[0] == '-') throw std::runtime_error("meta.dat: expected an integer, got '" + t + "'");
        return v;
    }
    double f64() {
        const std::string t = next();
        char* end = nullptr;
        const double v = std::strtod(t.c_str(), &end);
        if (t.empty() || *end) throw std::runtime_error("meta.dat: expected a number, got '" + t + "'");
        return v;
    }
};

}  // namespace

std::string encode_meta(const Meta& m) {
    std::ostringstream o;
    o << kSigLen << ' ' << kSignature << ' ' << kWriteLibraryVersion << ' ' << m.version;
    o << " 3";
    for (int d = 0; d < 3; ++d) o << ' ' << sci(m.box.init_xyz[d]);
    o << " 3";
    for (int d = 0; d < 3; ++d) o << ' ' << m.box.npoints[d];
    o << ' ' << sci(m.box.spacing);
    o << " 0 0 " << m.excluded.size() << ' ' << bucket_count_for(m.excluded.size()) << " 0";
    for (int64_t a : m.excluded) o << ' ' << a;
    o << '\n';
    return o.str();
}

Meta decode_meta(const std::string& text) {
    Tokens t(text);
    if (t.u64() != kSigLen || t.next() != kSignature) throw std::runtime_error("meta.dat is not a Boost text archive");
    const uint64_t lib = t.u64();
    if (lib < 8) throw std::runtime_error("Boost archive library version " + std::to_string(lib) + " is older than 8");
    Meta m;
    m.version = t.u64();
    if (m.version != kFormatVersion) return m;  // the caller reports the reference's message
    if (t.u64() != 3) throw std::runtime_error("meta.dat: init_xyz is not 3 values");
    for (int d = 0; d < 3; ++d) m.box.init_xyz[d] = t.f64();
    if (t.u64() != 3) throw std::runtime_error("meta.dat: npoints is not 3 values");
    for (int d = 0; d < 3; ++d) {
        const uint64_t n = t.u64();
        if (n < 2 || n > static_cast<uint64_t>(std::numeric_limits<int32_t>::max()))
            throw std::runtime_error("meta.dat: points per axis out of range");
        m.box.npoints[d] = static_cast<int32_t>(n);
    }
    m.box.spacing = t.f64();
    if (!(m.box.spacing > 0.0) || !std::isfinite(m.box.spacing)) throw std::runtime_error("meta.dat: bad spacing");
    const uint64_t tracking = t.u64(), version = t.u64();
    if (tracking > 1 || version != 0) throw std::runtime_error("meta.dat: unexpected class preamble of the atom set");
    const uint64_t count = t.u64();
    t.u64();  // bucket count
    t.u64();  // item version
    if (count > (1u << 30)) throw std::runtime_error("meta.dat: excluded atom count out of range");
    m.excluded.reserve(count);
    for (uint64_t i = 0; i < count; ++i) m.excluded.push_back(static_cast<int64_t>(t.u64()));
    return m;
}

}  // namespace mapcache
}  // namespace pxd

// ------------------------------------------------------------------ C ABI (host only)

extern "C" {

int64_t pxd_bdg_encode(const double* records, int64_t n_points, int32_t value_bytes, uint8_t* out,
                       int64_t out_capacity) {
    if (n_points < 0 || (n_points > 0 && !records) || (value_bytes != 8 && value_bytes != 4)) return -PXD_ERR_INVALID;
    try {
        const std::vector<uint8_t> b = pxd::mapcache::encode_bdg(records, static_cast<size_t>(n_points), value_bytes);
        const int64_t n = static_cast<int64_t>(b.size());
        if (out && out_capacity >= n) std::memcpy(out, b.data(), b.size());
        return n;
    } catch (...) {
        return -PXD_ERR_NOMEM;
    }
}

int64_t pxd_bdg_decode(const uint8_t* data, int64_t size, double* records, int64_t capacity_points,
                       int32_t* value_bytes) {
    if (!data || size < 0) return -PXD_ERR_INVALID;
    try {
        int vb = 0;
        const std::vector<double> rec = pxd::mapcache::decode_bdg(data, static_cast<size_t>(size), &vb);
        const int64_t n = static_cast<int64_t>(rec.size() / 4);
        if (records && capacity_points >= n) std::memcpy(records, rec.data(), rec.size() * sizeof(double));
        if (value_bytes) *value_bytes = vb;
        return n;
    } catch (const std::bad_alloc&) {
        return -PXD_ERR_NOMEM;
    } catch (...) {
        return -PXD_ERR_IO;
    }
}

int64_t pxd_meta_encode(const pxd_box* box, const int64_t* excluded, int64_t n_excluded, char* out,
                        int64_t out_capacity) {
    if (!box || n_excluded < 0 || (n_excluded > 0 && !excluded)) return -PXD_ERR_INVALID;
    try {
        pxd::mapcache::Meta m;
        m.box = *box;
        m.excluded.assign(excluded, excluded + n_excluded);
        const std::string s = pxd::mapcache::encode_meta(m);
        const int64_t n = static_cast<int64_t>(s.size());
        if (out && out_capacity >= n + 1) std::memcpy(out, s.c_str(), s.size() + 1);
        return n;
    } catch (...) {
        return -PXD_ERR_NOMEM;
    }
}

int64_t pxd_meta_decode(const char* text, int64_t size, pxd_box* box, uint64_t* version, int64_t* excluded,
                        int64_t capacity) {
    if (!text || size < 0) return -PXD_ERR_INVALID;
    try {
        const pxd::mapcache::Meta m = pxd::mapcache::decode_meta(std::string(text, static_cast<size_t>(size)));
        if (version) *version = m.version;
        if (box) *box = m.box;
        const int64_t n = static_cast<int64_t>(m.excluded.size());
        if (excluded && capacity >= n) std::memcpy(excluded, m.excluded.data(), m.excluded.size() * sizeof(int64_t));
        return n;
    } catch (const std::bad_alloc&) {
        return -PXD_ERR_NOMEM;
    } catch (...) {
        return -PXD_ERR_IO;
    }
}

}  // extern "C"
