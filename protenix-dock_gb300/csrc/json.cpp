// JSON reader (see json.h): recursive descent over RFC 8259 with \uXXXX escapes turned
// into UTF-8; numbers through strtod.
#include "json.h"

#include <cstring>
#include <fstream>
#include <sstream>

namespace pxd {
namespace json {

namespace {

struct Parser {
    const char* p;
    const char* begin;
    const char* end;
    int depth = 0;

    [[noreturn]] void fail(const char* what) const {
        std::ostringstream oss;
        oss << "JSON parse error at byte " << (p - begin) << ": " << what;
        throw std::runtime_error(oss.str());
    }
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool eat(char c) {
        ws();
        if (p < end && *p == c) {
            ++p;
            return true;
        }
        return false;
    }
    void expect(char c) {
        if (!eat(c)) fail("unexpected character");
    }
    static void utf8(std::string& out, unsigned cp) {
        if (cp < 0x80) {
            out += static_cast<char>(cp);
        } else if (cp < 0x800) {
            out += static_cast<char>(0xC0 | (cp >> 6));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += static_cast<char>(0xE0 | (cp >> 12));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else {
            out += static_cast<char>(0xF0 | (cp >> 18));
            out += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        }
    }
    unsigned hex4() {
        if (end - p < 4) fail("short \\u escape");
        unsigned v = 0;
        for (int k = 0; k < 4; ++k, ++p) {
            const char c = *p;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= static_cast<unsigned>(c - '0');
            else if (c >= 'a' && c <= 'f') v |= static_cast<unsigned>(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= static_cast<unsigned>(c - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string string() {
        expect('"');
        std::string out;
        while (true) {
            if (p >= end) fail("unterminated string");
            const char c = *p++;
            if (c == '"') break;
            if (c != '\\') {
                out += c;
                continue;
            }
            if (p >= end) fail("unterminated escape");
            const char e = *p++;
            switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    unsigned cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        p += 2;
                        const unsigned lo = hex4();
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
        return out;
    }
    Value value() {
        if (++depth > 256) fail("nesting too deep");
        ws();
        if (p >= end) fail("unexpected end");
        Value v;
        const char c = *p;
        if (c == '{') {
            ++p;
            v.kind = Value::Object;
            if (!eat('}')) {
                do {
                    ws();
                    std::string key = string();
                    expect(':');
                    v.fields.emplace_back(std::move(key), value());
                } while (eat(','));
                expect('}');
            }
        } else if (c == '[') {
            ++p;
            v.kind = Value::Array;
            if (!eat(']')) {
                do {
                    v.items.push_back(value());
                } while (eat(','));
                expect(']');
            }
        } else if (c == '"') {
            v.kind = Value::String;
            v.str = string();
        } else if (c == 't' && end - p >= 4 && std::strncmp(p, "true", 4) == 0) {
            p += 4;
            v.kind = Value::Bool;
            v.b = true;
        } else if (c == 'f' && end - p >= 5 && std::strncmp(p, "false", 5) == 0) {
            p += 5;
            v.kind = Value::Bool;
        } else if (c == 'n' && end - p >= 4 && std::strncmp(p, "null", 4) == 0) {
            p += 4;
        } else {
            char* stop = nullptr;
            v.num = std::strtod(p, &stop);
            if (stop == p) fail("bad value");
            p = stop;
            v.kind = Value::Number;
        }
        --depth;
        return v;
    }
};

}  // namespace

Value parse(const std::string& text) {
    Parser ps{text.data(), text.data(), text.data() + text.size()};
    Value v = ps.value();
    ps.ws();
    if (ps.p != ps.end) ps.fail("trailing characters");
    return v;
}

Value parse_file(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Failed to open file: " + path);
    std::ostringstream ss;
    ss << in.rdbuf();
    return parse(ss.str());
}

}  // namespace json
}  // namespace pxd
