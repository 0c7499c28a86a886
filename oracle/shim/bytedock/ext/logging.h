// Test-infrastructure shim for the reference oracle build: it stands in for the
// reference's Boost.Log header (engine/include/bytedock/ext/logging.h) and discards
// every log record. The oracle is only called as a checker, so no log is wanted.
#pragma once

#include <memory>
#include <ostream>
#include <string>

#include "bytedock/ext/counter.h"

namespace bytedock {

struct shim_null_log {
    template <class T>
    shim_null_log& operator<<(const T&) { return *this; }
    shim_null_log& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};

struct sink_t {};

#define LOG_TRACE ::bytedock::shim_null_log()
#define LOG_DEBUG ::bytedock::shim_null_log()
#define LOG_INFO ::bytedock::shim_null_log()
#define LOG_WARNING ::bytedock::shim_null_log()
#define LOG_ERROR ::bytedock::shim_null_log()
#define LOG_FATAL ::bytedock::shim_null_log()
#define LOG_TELL_COUNTER(category)
#define LOG_TELL_THREAD_ID(...)

std::shared_ptr<sink_t> enable_global_logging(const std::string& path, int verbosity);
void disable_sink(std::shared_ptr<sink_t> sink, bool deregister = true);

}  // namespace bytedock

namespace boost {
using std::shared_ptr;
}
