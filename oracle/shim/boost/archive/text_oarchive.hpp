// Test-infrastructure shim for the reference oracle build: map save/restore is not
// exercised through the oracle, so this archive accepts and ignores everything.
#pragma once
#include <iosfwd>
namespace boost {
namespace archive {
class text_oarchive {
public:
    template <class S> explicit text_oarchive(S&) {}
    template <class T> text_oarchive& operator<<(const T&) { return *this; }
    template <class T> text_oarchive& operator>>(T&) { return *this; }
    template <class T> text_oarchive& operator&(T&) { return *this; }
};
}  // namespace archive
}  // namespace boost
