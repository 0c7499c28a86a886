// Test-infrastructure shim for the reference oracle build: boost::lexical_cast
// for the one use the reference parser makes (string key -> index, data.cpp:428).
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>
namespace boost {
class bad_lexical_cast : public std::bad_cast {};
template <class T, class S>
T lexical_cast(const S& src) {
    std::stringstream ss;
    ss << src;
    T out;
    ss >> out;
    if (ss.fail()) throw bad_lexical_cast();
    return out;
}
}  // namespace boost
