// Test-infrastructure shim: host helpers that the reference engine declares in
// engine/include/bytedock/ext/{pfile,logging}.h and engine/include/bytedock/version.h.
// The reference's own definitions need Boost.Log, Boost.Filesystem and an object-store
// SDK, none of which exist here, so plain-file versions stand in. Only the oracle
// library (built from the reference sources for parity checks) links this file.
#include <fstream>
#include <memory>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <limits.h>

#include "bytedock/ext/logging.h"
#include "bytedock/ext/pfile.h"
#include "bytedock/lib/error.h"

namespace bytedock {

const char* VERSION_STR = "ProtenixDock reference (oracle build)";

uintmax_t get_file_length(const std::string& path) {
    struct stat st;
    if (::stat(path.c_str(), &st) != 0) throw file_system_error("missing file: " + path);
    return static_cast<uintmax_t>(st.st_size);
}

std::shared_ptr<std::istream> open_for_read(const std::string& path) {
    auto in = std::make_shared<std::ifstream>(path);
    if (!in->good()) throw file_system_error("Failed to open file: " + path);
    return in;
}

std::shared_ptr<std::ostream> open_for_write(const std::string& path) {
    auto out = std::make_shared<std::ofstream>(path);
    if (!out->good()) throw file_system_error("Failed to create file: " + path);
    return out;
}

std::unique_ptr<std::ostream> open_for_append(const std::string& path) {
    std::unique_ptr<std::ostream> out(new std::ofstream(path, std::ios::app));
    return out;
}

bool is_file(const std::string& path) {
    struct stat st;
    return ::stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

void create_directory(const std::string& path) {
    std::string acc;
    for (size_t i = 0; i <= path.size(); ++i) {
        if (i == path.size() || path[i] == '/') {
            if (!acc.empty()) ::mkdir(acc.c_str(), 0755);
        }
        if (i < path.size()) acc += path[i];
    }
}

std::string get_executable_path() {
    char buf[PATH_MAX];
    ssize_t n = ::readlink("/proc/self/exe", buf, sizeof(buf) - 1);
    if (n < 0) return "";
    buf[n] = 0;
    return std::string(buf);
}

std::shared_ptr<sink_t> enable_global_logging(const std::string&, int) {
    return std::make_shared<sink_t>();
}

void disable_sink(std::shared_ptr<sink_t>, bool) {}

}  // namespace bytedock
