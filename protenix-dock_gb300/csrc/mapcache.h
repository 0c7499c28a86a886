// The reference's receptor-map cache files (receptor_cache::save / restore,
// engine/src/core/grid.cpp:305-431): one Boost.Serialization binary archive per map,
// <tag>.bdg, holding the map's std::vector<val_and_grad> (grid.h:54-57, grid.cpp:88-99),
// and a Boost text archive meta.dat holding the format version 20241030, the box origin,
// the points per axis, the spacing and the excluded (movable) receptor atoms, written
// last as the completion flag. Host code only; errors are std::runtime_error.
#ifndef PXD_MAPCACHE_H_
#define PXD_MAPCACHE_H_

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pxdock_gb300.h"

namespace pxd {
namespace mapcache {

// kFormatVersion (grid.cpp:307)
constexpr uint64_t kFormatVersion = 20241030;
// The Boost archive library version this writer stamps: the oldest layout it writes is
// the one every Boost >= 1.44 (library version 8) reads, and 17 is Boost 1.68 - 1.75,
// which the reference's Boost >= 1.72 reads as well.
constexpr int kWriteLibraryVersion = 17;

// records: n points x {E, dE/dx, dE/dy, dE/dz}; value_bytes 8 (the reference's default
// double build) or 4 (its float build). Returns the archive's bytes.
std::vector<uint8_t> encode_bdg(const double* records, size_t n_points, int value_bytes);
// Parses one .bdg archive; returns the points and sets value_bytes (8 or 4), which is
// told apart by the archive's length.
std::vector<double> decode_bdg(const uint8_t* data, size_t size, int* value_bytes);

struct Meta {
    uint64_t version = kFormatVersion;
    pxd_box box{};
    std::vector<int64_t> excluded;
};
std::string encode_meta(const Meta& meta);
Meta decode_meta(const std::string& text);

}  // namespace mapcache
}  // namespace pxd

#endif  // PXD_MAPCACHE_H_
