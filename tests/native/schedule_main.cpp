// Test harness: reads term lists from stdin and prints the conflict-free schedule
// that the library packs on the device (protenix-dock_gb300/csrc/schedule.h).
//   input:  K n_atoms n_terms, then n_terms lines of K atom indices
//   output: the schedule, one slot per line (term index | 1<<30 when reversed, or -1)
#include <cstdio>
#include <vector>

#include "schedule.h"

template <int K>
static int run(int n_atoms, int n_terms) {
    std::vector<std::array<int, K>> terms(n_terms);
    for (auto& t : terms)
        for (int k = 0; k < K; ++k)
            if (std::scanf("%d", &t[k]) != 1) return 2;
    for (int s : pxd::schedule_rounds<K>(terms, n_atoms)) std::printf("%d\n", s);
    return 0;
}

int main() {
    int K, n_atoms, n_terms;
    if (std::scanf("%d %d %d", &K, &n_atoms, &n_terms) != 3) return 2;
    switch (K) {
        case 2: return run<2>(n_atoms, n_terms);
        case 3: return run<3>(n_atoms, n_terms);
        case 4: return run<4>(n_atoms, n_terms);
        default: return 2;
    }
}
