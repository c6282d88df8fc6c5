// Checks gb300::CopyPool (solana-perf-libs_gb300/csrc/host_copy.h) on the
// host: random piece layouts, below and above the parallel threshold, from
// several caller threads at once (callers that find the pool busy copy
// alone).  Every destination byte must equal its source and bytes between
// pieces must stay untouched.  Prints "ok" and exits 0 on success.
#include <cstdio>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "host_copy.h"

static bool one_case(std::mt19937_64& rng, size_t total_max) {
    std::uniform_int_distribution<size_t> npieces(1, 40);
    const size_t n = npieces(rng);
    std::vector<size_t> lens(n);
    size_t total = 0;
    for (auto& l : lens) {
        l = std::uniform_int_distribution<size_t>(0, total_max / n)(rng);
        total += l;
    }
    std::vector<unsigned char> src(total + 1), dst(total + 64 * n + 1, 0xA5);
    for (auto& b : src) b = (unsigned char)rng();
    std::vector<gb300::CopyPiece> pcs;
    std::vector<size_t> doff;
    size_t so = 0, d = 0;
    for (size_t i = 0; i < n; i++) {
        d += rng() % 64;                          // gaps that must stay untouched
        pcs.push_back({dst.data() + d, src.data() + so, lens[i]});
        doff.push_back(d);
        so += lens[i];
        d += lens[i];
    }
    gb300::CopyPool::copy(pcs.data(), pcs.size());
    std::vector<char> covered(dst.size(), 0);
    so = 0;
    for (size_t i = 0; i < n; i++) {
        if (memcmp(dst.data() + doff[i], src.data() + so, lens[i]) != 0) return false;
        memset(covered.data() + doff[i], 1, lens[i]);
        so += lens[i];
    }
    for (size_t k = 0; k < dst.size(); k++)
        if (!covered[k] && dst[k] != 0xA5) return false;
    return true;
}

int main() {
    std::vector<std::thread> th;
    std::vector<int> ok(4, 1);
    for (int t = 0; t < 4; t++)
        th.emplace_back([t, &ok] {
            std::mt19937_64 rng(1234 + t);
            for (int k = 0; k < 24 && ok[t]; k++)
                ok[t] = one_case(rng, k % 3 == 0 ? (64u << 10) : (24u << 20));
        });
    for (auto& x : th) x.join();
    for (int v : ok)
        if (!v) {
            printf("mismatch\n");
            return 1;
        }
    printf("ok\n");
    return 0;
}
