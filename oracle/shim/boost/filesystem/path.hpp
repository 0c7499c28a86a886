// Test-infrastructure shim for the reference oracle build: the few
// boost::filesystem::path members the reference engine calls.
#pragma once
#include <string>
namespace boost {
namespace filesystem {
class path {
public:
    path() {}
    path(const std::string& s) : s_(s) {}
    path(const char* s) : s_(s) {}
    const std::string& string() const { return s_; }
    path operator/(const path& other) const {
        if (s_.empty()) return other;
        if (s_.back() == '/') return path(s_ + other.s_);
        return path(s_ + "/" + other.s_);
    }
    path parent_path() const {
        size_t p = s_.find_last_of('/');
        if (p == std::string::npos) return path();
        return path(s_.substr(0, p));
    }
    path filename() const {
        size_t p = s_.find_last_of('/');
        return path(p == std::string::npos ? s_ : s_.substr(p + 1));
    }
    path stem() const {
        std::string f = filename().string();
        size_t d = f.find_last_of('.');
        if (d == std::string::npos || f == "." || f == "..") return path(f);
        return path(f.substr(0, d));
    }
private:
    std::string s_;
};
}  // namespace filesystem
}  // namespace boost
