// Test harness: parses the JSON document on stdin with the library's reader
// (protenix-dock_gb300/csrc/json.cpp) and prints it back in a canonical form
// (keys in file order, numbers with 17 significant digits).
#include <cstdio>
#include <iostream>
#include <sstream>

#include "json.h"

static void dump(const pxd::json::Value& v) {
    using K = pxd::json::Value;
    switch (v.kind) {
        case K::Null: std::printf("null"); break;
        case K::Bool: std::printf(v.b ? "true" : "false"); break;
        case K::Number: std::printf("%.17g", v.num); break;
        case K::String:
            std::printf("\"");
            for (unsigned char c : v.str) std::printf(c < 0x20 || c == '"' || c == '\\' ? "\\u%04x" : "%c", c);
            std::printf("\"");
            break;
        case K::Array:
            std::printf("[");
            for (size_t i = 0; i < v.items.size(); ++i) {
                if (i) std::printf(",");
                dump(v.items[i]);
            }
            std::printf("]");
            break;
        case K::Object:
            std::printf("{");
            for (size_t i = 0; i < v.fields.size(); ++i) {
                if (i) std::printf(",");
                std::printf("\"%s\":", v.fields[i].first.c_str());
                dump(v.fields[i].second);
            }
            std::printf("}");
            break;
    }
}

int main() {
    std::stringstream ss;
    ss << std::cin.rdbuf();
    try {
        dump(pxd::json::parse(ss.str()));
        std::printf("\n");
        return 0;
    } catch (std::exception& e) {
        std::printf("ERROR %s\n", e.what());
        return 1;
    }
}
