// Conflict-free term scheduling for the warp-per-pose force field (host code).
//
// A warp evaluates one term per lane per round and scatters the gradient of the
// atom in position k of each term into gradient array k (shared memory, one array
// per position). A round is conflict-free when, for every position, its terms name
// distinct atoms there. Every term kind of the force field is unchanged when its
// atom list is reversed (bonds and pairs i-j, angles i-j-k, dihedrals i-j-k-l), so
// each term may also be placed reversed. A slot of the schedule is a term index with
// bit 30 set for "reversed", or -1 for an empty lane.
#ifndef PXD_SCHEDULE_H_
#define PXD_SCHEDULE_H_

#include <stdint.h>

#include <algorithm>
#include <array>
#include <vector>

namespace pxd {

constexpr int kLanes = 32;
constexpr int kReversed = 1 << 30;

// Small deterministic generator for the shuffles of the packing search (xorshift64).
struct Shuffler {
    uint64_t s = 0x9e3779b97f4a7c15ull;
    uint32_t next() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return static_cast<uint32_t>(s >> 32);
    }
};

template <int K>
struct RoundPacker {
    const std::vector<std::array<int, K>>& terms;
    int n_atoms;

    // Places term t into round r if its atoms are free there, in either orientation.
    bool place(std::vector<uint8_t>& used, std::vector<int>& round_of, int t, int r) const {
        for (int rev = 0; rev < 2; ++rev) {
            bool ok = true;
            for (int k = 0; k < K && ok; ++k) {
                const int a = terms[t][rev ? K - 1 - k : k];
                ok = !used[static_cast<size_t>(k) * n_atoms + a];
            }
            if (!ok) continue;
            for (int k = 0; k < K; ++k) {
                const int a = terms[t][rev ? K - 1 - k : k];
                used[static_cast<size_t>(k) * n_atoms + a] = 1;
            }
            round_of[t] = r | (rev ? kReversed : 0);
            return true;
        }
        return false;
    }

    // First-fit: fill round after round in term order; returns the number of rounds.
    int first_fit(std::vector<int>& round_of) const {
        const int n = static_cast<int>(terms.size());
        std::vector<char> done(n, 0);
        std::vector<uint8_t> used;
        int left = n, r = 0;
        while (left > 0) {
            used.assign(static_cast<size_t>(K) * n_atoms, 0);
            int filled = 0;
            for (int t = 0; t < n && filled < kLanes; ++t) {
                if (done[t]) continue;
                if (place(used, round_of, t, r)) {
                    done[t] = 1;
                    ++filled;
                    --left;
                }
            }
            ++r;
        }
        return r;
    }

    // Balanced: R rounds, each term (in `order`) into the least-filled round that takes it.
    bool balanced(int R, const std::vector<int>& order, std::vector<int>& round_of) const {
        std::vector<std::vector<uint8_t>> used(R, std::vector<uint8_t>(static_cast<size_t>(K) * n_atoms, 0));
        std::vector<int> fill(R, 0), by_fill(R);
        for (int t : order) {
            for (int r = 0; r < R; ++r) by_fill[r] = r;
            std::stable_sort(by_fill.begin(), by_fill.end(), [&](int a, int b) { return fill[a] < fill[b]; });
            bool ok = false;
            for (int r : by_fill) {
                if (fill[r] >= kLanes) break;
                if (place(used[r], round_of, t, r)) {
                    ++fill[r];
                    ok = true;
                    break;
                }
            }
            if (!ok) return false;
        }
        return true;
    }
};

// Orders terms into as few conflict-free rounds of 32 as the search finds: first-fit,
// then balanced packings into fewer rounds (down to ceil(n / 32)) over seeded shuffles,
// within a bounded number of placements. Deterministic.
template <int K>
std::vector<int> schedule_rounds(const std::vector<std::array<int, K>>& terms, int n_atoms) {
    const int n = static_cast<int>(terms.size());
    if (n == 0) return {};
    RoundPacker<K> pk{terms, n_atoms};
    std::vector<int> best(n), trial(n);
    int best_r = pk.first_fit(best);
    const int lower = (n + kLanes - 1) / kLanes;
    std::vector<int> order(n);
    for (int t = 0; t < n; ++t) order[t] = t;
    Shuffler rng;
    const long budget = 4000000;
    long spent = 0;
    for (int R = lower; R < best_r && spent < budget; ++R) {
        bool found = false;
        for (int attempt = 0; attempt < 32 && spent < budget; ++attempt) {
            if (attempt > 0)
                for (int t = n - 1; t > 0; --t) std::swap(order[t], order[rng.next() % (t + 1)]);
            spent += static_cast<long>(n) * R;
            if (pk.balanced(R, order, trial)) {
                best.swap(trial);
                best_r = R;
                found = true;
                break;
            }
        }
        if (found) break;
    }
    std::vector<std::vector<int>> rounds(best_r);
    for (int t = 0; t < n; ++t) rounds[best[t] & ~kReversed].push_back(t | (best[t] & kReversed));
    std::vector<int> out;
    out.reserve(static_cast<size_t>(best_r) * kLanes);
    for (auto& r : rounds) {
        for (int v : r) out.push_back(v);
        for (size_t k = r.size(); k < static_cast<size_t>(kLanes); ++k) out.push_back(-1);
    }
    return out;
}

// The atoms of scheduled slot s (a term index, possibly reversed) in lane order.
template <int K>
std::array<int, K> slot_atoms(const std::vector<std::array<int, K>>& terms, int s) {
    const std::array<int, K>& t = terms[s & ~kReversed];
    if (!(s & kReversed)) return t;
    std::array<int, K> r;
    for (int k = 0; k < K; ++k) r[k] = t[K - 1 - k];
    return r;
}

}  // namespace pxd

#endif  // PXD_SCHEDULE_H_
