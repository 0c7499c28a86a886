// Test-infrastructure shim for the reference oracle build: a silent progress display.
#pragma once
namespace boost {
class progress_display {
public:
    explicit progress_display(unsigned long) {}
    unsigned long operator++() { return ++n_; }
    unsigned long operator+=(unsigned long k) { return n_ += k; }
private:
    unsigned long n_ = 0;
};
}  // namespace boost
