// Test-infrastructure shim: a small JSON reader producing the ordered property tree of
// ptree.hpp, with Boost's conventions (array items have empty keys, scalars are kept as
// their source text). Only the reference oracle build uses it.
#pragma once

#include <cctype>
#include <istream>
#include <iterator>
#include <string>

#include "boost/property_tree/ptree.hpp"

namespace boost {
namespace property_tree {

class json_parser_error : public ptree_error {
public:
    explicit json_parser_error(const std::string& m) : ptree_error("json: " + m) {}
};

namespace json_detail {

struct reader {
    const std::string& s;
    size_t i = 0;
    explicit reader(const std::string& src) : s(src) {}

    void ws() {
        while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
    }
    char peek() {
        ws();
        if (i >= s.size()) throw json_parser_error("unexpected end");
        return s[i];
    }
    void expect(char c) {
        if (peek() != c) throw json_parser_error(std::string("expected ") + c);
        ++i;
    }
    std::string str() {
        expect('"');
        std::string out;
        while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\') {
                ++i;
                if (i >= s.size()) break;
                char e = s[i];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        unsigned code = std::stoul(s.substr(i + 1, 4), nullptr, 16);
                        i += 4;
                        if (code < 0x80) {
                            out += static_cast<char>(code);
                        } else if (code < 0x800) {
                            out += static_cast<char>(0xC0 | (code >> 6));
                            out += static_cast<char>(0x80 | (code & 0x3F));
                        } else {
                            out += static_cast<char>(0xE0 | (code >> 12));
                            out += static_cast<char>(0x80 | ((code >> 6) & 0x3F));
                            out += static_cast<char>(0x80 | (code & 0x3F));
                        }
                        break;
                    }
                    default: out += e;
                }
                ++i;
            } else {
                out += s[i++];
            }
        }
        expect('"');
        return out;
    }
    void value(ptree& node) {
        char c = peek();
        if (c == '{') {
            ++i;
            if (peek() == '}') { ++i; return; }
            while (true) {
                std::string key = str();
                expect(':');
                ptree child;
                value(child);
                node.push_back(key, child);
                char d = peek();
                ++i;
                if (d == '}') return;
                if (d != ',') throw json_parser_error("bad object");
            }
        } else if (c == '[') {
            ++i;
            if (peek() == ']') { ++i; return; }
            while (true) {
                ptree child;
                value(child);
                node.push_back("", child);
                char d = peek();
                ++i;
                if (d == ']') return;
                if (d != ',') throw json_parser_error("bad array");
            }
        } else if (c == '"') {
            node.data() = str();
        } else {
            size_t start = i;
            while (i < s.size() && s[i] != ',' && s[i] != '}' && s[i] != ']' &&
                   !std::isspace(static_cast<unsigned char>(s[i]))) ++i;
            node.data() = s.substr(start, i - start);
        }
    }
};

}  // namespace json_detail

inline void read_json(std::istream& in, ptree& pt) {
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    json_detail::reader r(text);
    ptree root;
    r.value(root);
    pt = root;
}

}  // namespace property_tree
}  // namespace boost
