// Test-infrastructure shim for the reference oracle build.
#pragma once
#include <sys/stat.h>
#include "boost/filesystem/path.hpp"
namespace boost {
namespace filesystem {
inline bool exists(const path& p) {
    struct stat st;
    return ::stat(p.string().c_str(), &st) == 0;
}
}  // namespace filesystem
}  // namespace boost
