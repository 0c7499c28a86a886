// Test-infrastructure shim: a minimal ordered property tree with the subset of the
// Boost.PropertyTree interface that the reference engine's parsers call
// (engine/src/core/data.cpp:31-520, engine/src/core/factory.cpp:31-212).
// It exists only so the reference sources compile in place as the oracle library;
// nothing in the product links it.
#pragma once

#include <cstdlib>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace boost {
namespace property_tree {

class ptree_error : public std::runtime_error {
public:
    explicit ptree_error(const std::string& m) : std::runtime_error(m) {}
};
class ptree_bad_path : public ptree_error {
public:
    explicit ptree_bad_path(const std::string& m) : ptree_error("No such node (" + m + ")") {}
};
class ptree_bad_data : public ptree_error {
public:
    explicit ptree_bad_data(const std::string& m) : ptree_error("conversion of data failed (" + m + ")") {}
};

namespace detail {
template <class T>
struct convert {
    static T from(const std::string& s) {
        std::istringstream iss(s);
        T v;
        iss >> v;
        if (iss.fail()) throw ptree_bad_data(s);
        return v;
    }
};
template <>
struct convert<std::string> {
    static std::string from(const std::string& s) { return s; }
};
template <>
struct convert<double> {
    static double from(const std::string& s) {
        char* end = nullptr;
        double v = std::strtod(s.c_str(), &end);
        if (end == s.c_str()) throw ptree_bad_data(s);
        return v;
    }
};
template <>
struct convert<float> {
    static float from(const std::string& s) { return static_cast<float>(convert<double>::from(s)); }
};
template <>
struct convert<unsigned long> {
    static unsigned long from(const std::string& s) {
        char* end = nullptr;
        unsigned long v = std::strtoul(s.c_str(), &end, 10);
        if (end == s.c_str()) throw ptree_bad_data(s);
        return v;
    }
};
}  // namespace detail

class ptree {
public:
    typedef std::pair<const std::string, ptree> value_type;
    typedef std::vector<std::pair<std::string, ptree> > container;
    typedef container::iterator iterator;
    typedef container::const_iterator const_iterator;

    ptree() {}
    explicit ptree(const std::string& data) : data_(data) {}

    size_t size() const { return children_.size(); }
    bool empty() const { return children_.empty(); }
    iterator begin() { return children_.begin(); }
    iterator end() { return children_.end(); }
    const_iterator begin() const { return children_.begin(); }
    const_iterator end() const { return children_.end(); }

    const std::string& data() const { return data_; }
    std::string& data() { return data_; }

    ptree& push_back(const std::string& key, const ptree& child) {
        children_.emplace_back(key, child);
        return children_.back().second;
    }

    size_t count(const std::string& key) const {
        size_t n = 0;
        for (auto& kv : children_) n += (kv.first == key);
        return n;
    }

    const ptree* find_path(const std::string& path) const {
        const ptree* node = this;
        size_t start = 0;
        while (true) {
            size_t dot = path.find('.', start);
            std::string key = path.substr(start, dot == std::string::npos ? std::string::npos : dot - start);
            const ptree* next = nullptr;
            for (auto& kv : node->children_) {
                if (kv.first == key) { next = &kv.second; break; }
            }
            if (!next) return nullptr;
            node = next;
            if (dot == std::string::npos) return node;
            start = dot + 1;
        }
    }

    const ptree& get_child(const std::string& path) const {
        const ptree* p = find_path(path);
        if (!p) throw ptree_bad_path(path);
        return *p;
    }

    template <class T>
    T get_value() const { return detail::convert<T>::from(data_); }

    template <class T>
    T get(const std::string& path) const { return get_child(path).get_value<T>(); }

    template <class T>
    T get(const std::string& path, const T& default_value) const {
        const ptree* p = find_path(path);
        if (!p) return default_value;
        return p->get_value<T>();
    }

    std::string get(const std::string& path, const char* default_value) const {
        const ptree* p = find_path(path);
        if (!p) return std::string(default_value);
        return p->data_;
    }

private:
    std::string data_;
    container children_;
};

}  // namespace property_tree
}  // namespace boost
