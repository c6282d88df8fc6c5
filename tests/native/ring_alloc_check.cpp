// Checks gb300::RingAlloc (solana-perf-libs_gb300/csrc/ring_alloc.h), the
// served loop's ring allocator, on the host: random sequences of
// allocations (sizes up to the capacity, alignments dividing it) and
// releases in random order.  At every step the live allocations must occupy
// disjoint physical ranges inside the buffer (contiguous mode) or disjoint
// sets of units (wrapping mode) and respect their alignment, and space must
// come back: after everything is released a full-capacity allocation
// succeeds.  Prints "ok" and exits 0 on success.
#include <cstdio>
#include <random>
#include <vector>

#include "ring_alloc.h"

namespace {

struct Live {
    uint64_t vpos, n, id;
};

bool check_disjoint(const std::vector<Live>& live, uint64_t cap, bool contiguous) {
    std::vector<int> used(cap, 0);
    for (const Live& l : live) {
        const uint64_t p = l.vpos % cap;
        if (contiguous && p + l.n > cap) return false;
        for (uint64_t k = 0; k < l.n; k++) {
            const uint64_t u = (p + k) % cap;
            if (used[u]++) return false;
        }
    }
    return true;
}

bool run(uint64_t cap, bool contiguous, uint64_t seed) {
    std::mt19937_64 rng(seed);
    gb300::RingAlloc R(cap, contiguous);
    std::vector<Live> live;
    int fails = 0, allocs = 0;
    for (int step = 0; step < 20000; step++) {
        const bool do_alloc = live.empty() || (rng() % 100) < 55;
        if (do_alloc) {
            const uint64_t n = (rng() % 4 == 0) ? rng() % (cap + 1) : rng() % (cap / 8 + 1);
            uint64_t align = contiguous ? (1ull << (rng() % 9)) : 1;
            while (cap % align) align >>= 1;            // alignments divide the capacity
            uint64_t v = 0, id = 0;
            if (R.alloc(n, align, &v, &id)) {
                if (v % align) {
                    printf("FAIL alignment cap=%llu\n", (unsigned long long)cap);
                    return false;
                }
                live.push_back({v, n, id});
                allocs++;
                if (!check_disjoint(live, cap, contiguous)) {
                    printf("FAIL overlap cap=%llu contiguous=%d step=%d\n", (unsigned long long)cap, contiguous, step);
                    return false;
                }
            } else {
                fails++;
                if (n <= cap && live.empty()) {
                    printf("FAIL refused on an empty ring n=%llu\n", (unsigned long long)n);
                    return false;
                }
            }
        } else {
            const size_t k = rng() % live.size();
            if (!R.release(live[k].id)) {
                printf("FAIL release\n");
                return false;
            }
            live.erase(live.begin() + (long)k);
        }
    }
    for (const Live& l : live)
        if (!R.release(l.id)) return false;
    uint64_t v, id;
    if (!R.empty() || !R.alloc(cap, 1, &v, &id)) {
        printf("FAIL space not returned\n");
        return false;
    }
    if (R.release(id + 1000)) return false;          // unknown id
    return allocs > 1000 && fails > 0;
}

}  // namespace

int main() {
    bool ok = true;
    for (uint64_t cap : {64ull, 1000ull, 4096ull})
        for (bool contiguous : {true, false})
            for (uint64_t seed = 1; seed <= 3; seed++) ok = ok && run(cap, contiguous, seed * 7919 + cap);
    if (!ok) return 1;
    printf("ok\n");
    return 0;
}
