// A small JSON reader for the engine's input files (receptor, ligand and scoring-function
// JSON as the reference engine reads them with boost::property_tree). Objects keep their
// key order: the reference walks some objects in file order (the receptor's rotor
// batches, the ligand's fragment traversal levels). Host code only.
#ifndef PXD_JSON_H_
#define PXD_JSON_H_

#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace pxd {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> items;                            // Array
    std::vector<std::pair<std::string, Value>> fields;   // Object, in file order

    bool is_null() const { return kind == Null; }
    bool has(const std::string& key) const { return find(key) != nullptr; }
    const Value* find(const std::string& key) const {
        for (auto& f : fields)
            if (f.first == key) return &f.second;
        return nullptr;
    }
    // member access that names the missing key, as property_tree's get_child does
    const Value& at(const std::string& key) const {
        const Value* v = find(key);
        if (!v) throw std::runtime_error("No such node (" + key + ")");
        return *v;
    }
    size_t size() const { return kind == Array ? items.size() : kind == Object ? fields.size() : 0; }
    double as_double() const {
        if (kind == Number) return num;
        if (kind == String) return std::strtod(str.c_str(), nullptr);  // property_tree reads "1.5" too
        if (kind == Bool) return b ? 1.0 : 0.0;
        throw std::runtime_error("JSON value is not a number");
    }
    long as_long() const { return static_cast<long>(as_double()); }
};

// Parses a whole document; throws std::runtime_error with the byte offset on bad input.
Value parse(const std::string& text);
Value parse_file(const std::string& path);

}  // namespace json
}  // namespace pxd

#endif  // PXD_JSON_H_
