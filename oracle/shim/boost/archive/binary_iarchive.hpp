// Test-infrastructure shim for the reference oracle build: map save/restore is not
// exercised through the oracle, so this archive accepts and ignores everything.
#pragma once
#include <iosfwd>
namespace boost {
namespace archive {
class binary_iarchive {
public:
    template <class S> explicit binary_iarchive(S&) {}
    template <class T> binary_iarchive& operator<<(const T&) { return *this; }
    template <class T> binary_iarchive& operator>>(T&) { return *this; }
    template <class T> binary_iarchive& operator&(T&) { return *this; }
};
}  // namespace archive
}  // namespace boost
