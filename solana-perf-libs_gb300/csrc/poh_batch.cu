// Ragged PoH batches: one persistent launch, longest chain first, lanes
// refilled from a shared queue.
//
// The plain form (poh.cu, the reference's poh_verify_kernel shape) gives each
// thread one entry for the whole launch: with counts spread over 1..1e6 a
// warp runs as long as its longest lane and, past 32 * (warps resident)
// entries, whole waves wait for the slowest warp of the previous wave.
// Here:
//   1. order    entries bucketed by bit length of num_hashes, longest
//               bucket first (three small kernels: histogram, scan, scatter);
//   2. persist  one warp per SM sub-partition; every lane whose chain is done
//               stores it and takes the next entry of the order (one
//               atomicAdd per warp per refill round, ranks by ballot), so the
//               warp keeps 32 chains in flight until the queue is empty.
//               Between refills all busy lanes step together for the
//               smallest remaining count among them, so the hashing loop
//               carries no per-step queue bookkeeping.
// Results are independent of which lane runs which entry.
//
// Scratch (PohBatchScratch) lives in caller-owned device memory:
// gb300_poh_batch_workspace_size(n) bytes.
#include <cuda_runtime.h>
#include "kernels.h"
#include "sha256_poh.cuh"

namespace {

constexpr int kBuckets = 65;   // bit length of num_hashes: 0..64

struct PohBatchScratch {
    uint32_t hist[kBuckets];
    uint32_t cursor[kBuckets];
    uint32_t next;              // queue head
    uint32_t choice;            // kPohAuto: 0 undecided, kChosePair or kChoseSingle
    uint64_t total, longest;    // kPohAuto: sum and maximum of the counts
    uint32_t order[1];          // n entries
};
constexpr uint32_t kChosePair = 1, kChoseSingle = 2;

__device__ __forceinline__ uint32_t bswap_u32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

__device__ __forceinline__ int bucket_of(uint64_t c) { return c ? 64 - __clzll((long long)c) : 0; }

// Bucket counts; with `totals`, also the sum and maximum of the counts
// (warp-reduced, one atomic per warp).
__global__ void poh_hist_kernel(const uint64_t* counts, uint64_t n, PohBatchScratch* s, bool totals) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t c = i < n ? counts[i] : 0;
    if (i < n) atomicAdd(&s->hist[bucket_of(c)], 1u);
    if (!totals) return;
    uint64_t sum = c, mx = c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        const uint64_t m = __shfl_down_sync(0xffffffffu, mx, o);
        mx = m > mx ? m : mx;
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&s->total), (unsigned long long)sum);
        atomicMax(reinterpret_cast<unsigned long long*>(&s->longest), (unsigned long long)mx);
    }
}

// kPohAuto: paired warps run a chain fastest (~1,900 cycles per hash on
// GB300) but hold two warps per 32 chains; single warps, four per
// sub-partition, take ~2,550 cycles per hash alone and share the ALU pipe at
// ~77.5 cycles per hash per sub-partition.  The shape with the smaller
// makespan estimate runs (single warps only when 10 % shorter), as the host
// forms decide from host counts.
//
// Both persistent kernels are enqueued, paired first, and steered through
// the queue rather than by a test in their code (an entry test in the
// paired kernel cost 0.5 % on GB300, its code being that sensitive to
// context): for single warps the queue head starts at n, so the paired
// kernel finds the queue empty and ends, and poh_requeue_kernel then resets
// it; for pairs the paired kernel drains the queue and the single-warp
// kernel finds it empty.
__global__ void poh_choose_kernel(PohBatchScratch* s, uint32_t sms, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double L = (double)s->longest, T = (double)s->total;
    const double pair = fmax(L * 1900.0, T * 1900.0 / (64.0 * sms));
    const double single = fmax(L * 2550.0, T * 77.5 / (4.0 * sms));
    s->choice = single < 0.9 * pair ? kChoseSingle : kChosePair;
    if (s->choice == kChoseSingle) s->next = n;
}

__global__ void poh_requeue_kernel(PohBatchScratch* s) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && s->choice == kChoseSingle) s->next = 0;
}

// single warp: cursor[b] = number of entries in buckets above b (longest first)
__global__ void poh_scan_kernel(PohBatchScratch* s) {
    if (threadIdx.x != 0) return;
    uint32_t run = 0;
    for (int b = kBuckets - 1; b >= 0; b--) {
        s->cursor[b] = run;
        run += s->hist[b];
    }
    s->next = 0;
}

__global__ void poh_scatter_kernel(const uint64_t* counts, uint64_t n, PohBatchScratch* s) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) s->order[atomicAdd(&s->cursor[bucket_of(counts[i])], 1u)] = (uint32_t)i;
}

__device__ __forceinline__ void load_entry(const uint8_t* hashes, uint64_t e, uint32_t w[8]) {
    const uint4* p = reinterpret_cast<const uint4*>(hashes + 32ull * e);
    uint4 lo = p[0], hi = p[1];
    w[0] = bswap_u32(lo.x); w[1] = bswap_u32(lo.y); w[2] = bswap_u32(lo.z); w[3] = bswap_u32(lo.w);
    w[4] = bswap_u32(hi.x); w[5] = bswap_u32(hi.y); w[6] = bswap_u32(hi.z); w[7] = bswap_u32(hi.w);
}

__device__ __forceinline__ void store_entry(uint8_t* hashes, uint64_t e, const uint32_t w[8]) {
    uint4* p = reinterpret_cast<uint4*>(hashes + 32ull * e);
    p[0] = make_uint4(bswap_u32(w[0]), bswap_u32(w[1]), bswap_u32(w[2]), bswap_u32(w[3]));
    p[1] = make_uint4(bswap_u32(w[4]), bswap_u32(w[5]), bswap_u32(w[6]), bswap_u32(w[7]));
}

struct HashWords {
    uint32_t v[8];
};

// The hashing loops of the persistent kernels are separate non-inlined
// functions.  Compiled inline, their schedule depended on the code around
// them: the single-warp loop ran at ~2,550 cycles per hash in a 32-thread
// block but ~3,150 in a 128-thread one, and the paired loop ~2,570 inside
// the queue loop against ~2,080 in a plain one-launch-per-batch kernel.
// Compiled alone they run at ~2,540 (single) and ~1,950 (paired) cycles.
static __device__ __noinline__ HashWords single_run(HashWords in, uint64_t r, uint32_t one) {
    const PohMul M(one);
    uint32_t w[8];
#pragma unroll
    for (int t = 0; t < 8; t++) w[t] = in.v[t];
#pragma unroll 1
    for (uint64_t k = 0; k < r; k++) poh_step_mix<0, 0, 0>(w, M);
    HashWords out;
#pragma unroll
    for (int t = 0; t < 8; t++) out.v[t] = w[t];
    return out;
}

// Where the persistent kernels' round warps run: per SM sub-partition (SM
// index x 4 + the warp slot's sub-partition), the round warps there now,
// and how many sub-partitions have at least one.  The served loop's
// signature service reads them (poh_round_warp_map) to prefer
// sub-partitions without one: a verify chain beside an ALU-bound round warp
// gets about half of the sub-partition's issue slots.  Diagnostic-grade
// placement (%warpid is the warp's slot when read); only a preference
// depends on it.
__device__ uint32_t g_poh_round_warps[kMaxServeSms * 4];
__device__ uint32_t g_poh_busy_slots;

__device__ __forceinline__ uint32_t poh_place_enter() {
    uint32_t smid, wid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(wid));
    const uint32_t slot = ((smid % kMaxServeSms) << 2) | (wid & 3u);
    if (atomicAdd(&g_poh_round_warps[slot], 1u) == 0u) atomicAdd(&g_poh_busy_slots, 1u);
    return slot;
}
__device__ __forceinline__ void poh_place_leave(uint32_t slot) {
    if (atomicSub(&g_poh_round_warps[slot], 1u) == 1u) atomicSub(&g_poh_busy_slots, 1u);
}

// BW independent warps per block.
template <int BW>
__global__ void __launch_bounds__(32 * BW) poh_persistent_kernel(uint8_t* hashes, const uint64_t* counts, uint32_t n,
                                                                 PohBatchScratch* s, uint32_t one) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t place = lane == 0 ? poh_place_enter() : 0u;
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint64_t rem = 0;
    uint32_t cur = 0xffffffffu;
    bool done = false;
    for (;;) {
        // refill every idle lane (several rounds when entries have count 0)
        for (;;) {
            const bool need = !done && rem == 0;
            const uint32_t mask = __ballot_sync(0xffffffffu, need);
            if (mask == 0) break;
            if (need && cur != 0xffffffffu) {
                store_entry(hashes, cur, w);
                cur = 0xffffffffu;
            }
            uint32_t base = 0;
            if (lane == (uint32_t)(__ffs(mask) - 1)) base = atomicAdd(&s->next, (uint32_t)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
            if (need) {
                const uint32_t k = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
                if (k >= n) {
                    done = true;
                } else {
                    cur = s->order[k];
                    load_entry(hashes, cur, w);
                    rem = counts[cur];
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        // run every busy lane until the first of them finishes: the inner
        // loop is then the plain chain loop, with no per-step bookkeeping
        uint64_t r = done ? ~0ull : rem;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t other = __shfl_xor_sync(0xffffffffu, r, o);
            r = other < r ? other : r;
        }
        if (!done) {
            HashWords h;
#pragma unroll
            for (int t = 0; t < 8; t++) h.v[t] = w[t];
            h = single_run(h, r, one);
#pragma unroll
            for (int t = 0; t < 8; t++) w[t] = h.v[t];
            rem -= r;
        }
    }
    if (lane == 0) poh_place_leave(place);
}

// Paired form: two warps per 32 lanes (the schedule warp computes the
// message schedule K[t] + W[t], t = 16..63, into shared memory while the
// round warp runs the 64 rounds: ~840 ALU instructions per hash on the round
// warp instead of ~1,330), inside the persistent longest-first loop.
// The round warp owns the queue: each refill round it stores finished
// chains, loads new ones and the step count r (the smallest remaining count
// among its busy lanes), and hands the current hash words and r to the
// schedule warp through shared memory at the pair's fifth barrier; then both
// run r hashes with the pair's barriers 1-4 per hash.  r == 0 means every
// lane is done and both warps leave together.  A block holds P pairs; pair
// p uses named barriers 6p+1 .. 6p+5 (64 threads each) and its own slices
// of the shared arrays, so pairs never wait on one another.
constexpr int kMaxPairsPerBlock = 2;
__shared__ uint32_t pair_kw[kMaxPairsPerBlock][48][32];   // K[t] + W[t], t = 16..63, per lane
__shared__ uint32_t pair_hout[kMaxPairsPerBlock][8][32];  // hash words, round warp -> schedule warp
__shared__ PohYield pair_yield;                           // poh_pair_yield_kernel's hint, set at its start

__device__ __forceinline__ uint32_t poh_ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Published signature chunks not yet claimed (head read first: head never
// passes the tail it was claimed under, so the difference is never negative).
__device__ __forceinline__ uint32_t poh_sig_backlog() {
    const uint32_t h = poh_ld_relaxed(pair_yield.head);
    return poh_ld_relaxed(pair_yield.tail) - h;
}

// Hashes the yielding form runs between looks at the backlog (~115 us).
constexpr uint64_t kYieldRun = 128;

// The round warp (every lane, converged) sleeps while the backlog stays at
// or above the threshold, its schedule warp waiting at the pair's barrier:
// at most kYieldNaps naps of ~16 us, then it runs kYieldRun hashes before it
// looks again.  The cap keeps PoH going under a backlog that lasts: with 256
// naps (~4 ms) PoH nearly stopped at 100 % of the served mix's peak, fell
// behind, and the signature p99 there doubled.
constexpr int kYieldNaps = 32;
__device__ __forceinline__ void poh_give_way() {
#pragma unroll 1
    for (int i = 0; i < kYieldNaps; i++) {
        if (poh_sig_backlog() < pair_yield.chunks) break;
        __nanosleep(16000);
    }
}

__device__ __forceinline__ uint32_t sched_s0(uint32_t x) { return POH_ROTR(x, 7) ^ POH_ROTR(x, 18) ^ (x >> 3); }
__device__ __forceinline__ uint32_t sched_s1(uint32_t x) { return POH_ROTR(x, 17) ^ POH_ROTR(x, 19) ^ (x >> 10); }

// Pair PI of its block (PI < 0: the pair index `pi` is a run-time value, so
// every pair of a block runs one copy of the code; with one copy per pair
// index the loops of a two-pair block outgrew the SM's instruction cache).
#define PAIR_IDX (PI >= 0 ? (uint32_t)PI : pi)

// round warp: r hashes of its 32 chains; a lane keeps its words after its
// first `lim` hashes (lim = 0 for a lane with no chain)
// Round additions issued on the multiply pipe as x * one + y (one == 1 at
// run time, so the compiler keeps the multiply-add): bit 2 h + K[t] + W[t],
// bit 0 e' = d + t1, bit 1 t2 = S0 + Maj, bit 3 a' = t1 + t2.  The round
// warp is bound by its ALU pipe; h + K + W is off the critical path, and
// moving it gained 2.0 % on GB300 (1,898 -> 1,860 cycles per hash).  The
// other additions are on the e / a dependency chains, where the multiply
// pipe's longer latency cost 3-20 %.
#ifndef POH_PAIR_MADD
#define POH_PAIR_MADD 4
#endif

template <int PI>
static __device__ __noinline__ HashWords pair_rounds(HashWords in, uint32_t lane, uint64_t r, uint64_t lim,
                                                     uint32_t pi, uint32_t one) {
    const uint32_t iv[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                            0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    uint32_t w[8];
#pragma unroll
    for (int t = 0; t < 8; t++) w[t] = in.v[t];
#pragma unroll 1
    for (uint64_t k = 0; k < r; k++) {
        uint32_t a = iv[0], b = iv[1], c = iv[2], d = iv[3], e = iv[4], f = iv[5], g = iv[6], h = iv[7];
#pragma unroll
        for (int t = 0; t < 64; t++) {
            if (t == 16 || t == 32 || t == 48) asm volatile("bar.sync %0, 64;" ::"r"(6 * PAIR_IDX + t / 16) : "memory");
            uint32_t x;
            if (t < 8) x = w[t] + poh_k(t);
            else if (t < 16) x = (t == 8 ? 0x80000000u : t == 15 ? 256u : 0u) + poh_k(t);
            else x = pair_kw[PAIR_IDX][t - 16][lane];
            const uint32_t S1 = POH_ROTR(e, 6) ^ POH_ROTR(e, 11) ^ POH_ROTR(e, 25);
            const uint32_t ch = (e & f) ^ (~e & g);
            const uint32_t S0 = POH_ROTR(a, 2) ^ POH_ROTR(a, 13) ^ POH_ROTR(a, 22);
            const uint32_t maj = (a & b) | (c & (a | b));
            const uint32_t hx = (POH_PAIR_MADD & 4) ? add_mul(h, x, one) : h + x;
            const uint32_t t1 = hx + S1 + ch;
            const uint32_t t2 = (POH_PAIR_MADD & 2) ? add_mul(S0, maj, one) : S0 + maj;
            h = g;
            g = f;
            f = e;
            e = (POH_PAIR_MADD & 1) ? add_mul(d, t1, one) : d + t1;
            d = c;
            c = b;
            b = a;
            a = (POH_PAIR_MADD & 8) ? add_mul(t1, t2, one) : t1 + t2;
        }
        const bool live = k < lim;
        w[0] = live ? iv[0] + a : w[0]; w[1] = live ? iv[1] + b : w[1];
        w[2] = live ? iv[2] + c : w[2]; w[3] = live ? iv[3] + d : w[3];
        w[4] = live ? iv[4] + e : w[4]; w[5] = live ? iv[5] + f : w[5];
        w[6] = live ? iv[6] + g : w[6]; w[7] = live ? iv[7] + h : w[7];
#pragma unroll
        for (int t = 0; t < 8; t++) pair_hout[PAIR_IDX][t][lane] = w[t];
        asm volatile("bar.sync %0, 64;" ::"r"(6 * PAIR_IDX + 4) : "memory");
    }
    HashWords out;
#pragma unroll
    for (int t = 0; t < 8; t++) out.v[t] = w[t];
    return out;
}

// schedule warp: the message schedule of r hashes, each from the hash words
// the round warp published at barrier 4 of the previous hash
template <int PI>
static __device__ __noinline__ void pair_schedule(HashWords in, uint32_t lane, uint64_t r, uint32_t pi) {
    uint32_t w[8];
#pragma unroll
    for (int t = 0; t < 8; t++) w[t] = in.v[t];
#pragma unroll 1
    for (uint64_t k = 0; k < r; k++) {
        uint32_t W[16];
#pragma unroll
        for (int t = 0; t < 8; t++) W[t] = w[t];
        W[8] = 0x80000000u;
#pragma unroll
        for (int t = 9; t < 15; t++) W[t] = 0;
        W[15] = 256u;
#pragma unroll
        for (int part = 0; part < 3; part++) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int t = 16 + part * 16 + j;
                const uint32_t x = W[t & 15] + sched_s0(W[(t - 15) & 15]) + W[(t - 7) & 15] + sched_s1(W[(t - 2) & 15]);
                W[t & 15] = x;
                pair_kw[PAIR_IDX][t - 16][lane] = x + poh_k(t);
            }
            asm volatile("bar.sync %0, 64;" ::"r"(6 * PAIR_IDX + 1 + part) : "memory");
        }
        asm volatile("bar.sync %0, 64;" ::"r"(6 * PAIR_IDX + 4) : "memory");
#pragma unroll
        for (int t = 0; t < 8; t++) w[t] = pair_hout[PAIR_IDX][t][lane];
    }
}

// s == nullptr: direct mode, no queue; the pair takes entries 32g .. 32g + 31
// once (g = its index in the grid), in the order given.
template <int PI, bool Y = false>
__device__ __forceinline__ void pair_persistent(uint8_t* hashes, const uint64_t* counts, uint32_t n,
                                                PohBatchScratch* s, uint64_t* run_len, uint32_t role, uint32_t pi,
                                                uint32_t direct_first, uint32_t one) {
    const uint32_t lane = threadIdx.x & 31u;
    HashWords w = {{0, 0, 0, 0, 0, 0, 0, 0}};
    uint64_t rem = 0;
    uint32_t cur = 0xffffffffu;
    uint32_t direct_k = direct_first + lane;
    bool done = false;
    for (;;) {
        if (role == 0) {
            for (;;) {
                const bool need = !done && rem == 0;
                const uint32_t mask = __ballot_sync(0xffffffffu, need);
                if (mask == 0) break;
                if (need && cur != 0xffffffffu) {
                    store_entry(hashes, cur, w.v);
                    cur = 0xffffffffu;
                }
                uint32_t k;
                if (s) {
                    uint32_t base = 0;
                    if (lane == (uint32_t)(__ffs(mask) - 1)) base = atomicAdd(&s->next, (uint32_t)__popc(mask));
                    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
                    k = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
                } else {
                    k = direct_k;
                    if (need) direct_k = 0xffffffffu;
                }
                if (need) {
                    if (k >= n) {
                        done = true;
                    } else {
                        cur = s ? s->order[k] : k;
                        load_entry(hashes, cur, w.v);
                        rem = counts[cur];
                    }
                }
            }
            uint64_t r = done ? ~0ull : rem;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t other = __shfl_xor_sync(0xffffffffu, r, o);
                r = other < r ? other : r;
            }
            if (r == ~0ull) r = 0;
            if (Y && r > 0) {
                // the yielding form runs at most kYieldRun hashes between
                // looks at the signature backlog (the hashing loops stay
                // those of the plain form)
                if (r > kYieldRun) r = kYieldRun;
                if (poh_sig_backlog() >= pair_yield.chunks) poh_give_way();
            }
#pragma unroll
            for (int t = 0; t < 8; t++) pair_hout[PAIR_IDX][t][lane] = w.v[t];
            if (lane == 0) *run_len = r;
        }
        asm volatile("bar.sync %0, 64;" ::"r"(6 * PAIR_IDX + 5) : "memory");
        const uint64_t r = *run_len;
        if (r == 0) break;
        if (role == 1) {
            HashWords h0;
#pragma unroll
            for (int t = 0; t < 8; t++) h0.v[t] = pair_hout[PAIR_IDX][t][lane];
            pair_schedule<PI>(h0, lane, r, pi);
        } else {
            w = pair_rounds<PI>(w, lane, r, done ? 0 : r, pi, one);
            if (!done) rem -= r;
        }
    }
}

// P pairs per block: warps 2p (rounds, queue) and 2p + 1 (schedule)
template <int P>
__global__ void __launch_bounds__(64 * P) poh_pair_persistent_kernel(uint8_t* hashes, const uint64_t* counts,
                                                                     uint32_t n, PohBatchScratch* s, uint32_t one) {
    static_assert(P >= 1 && P <= kMaxPairsPerBlock, "pairs per block");
    __shared__ uint64_t run_len[P];
    const uint32_t warp = threadIdx.x >> 5, pair = warp >> 1, role = warp & 1u;
    const uint32_t first = (blockIdx.x * P + pair) * 32u;   // direct mode only
    const bool counted = role == 0 && (threadIdx.x & 31u) == 0;  // the round warp's place
    const uint32_t place = counted ? poh_place_enter() : 0u;
    if (P == 1) pair_persistent<0>(hashes, counts, n, s, &run_len[0], role, 0, first, one);
    else pair_persistent<-1>(hashes, counts, n, s, &run_len[pair], role, pair, first, one);
    if (counted) poh_place_leave(place);
}

// The paired queue form that gives way to the signature service (PohYield).
__global__ void __launch_bounds__(64) poh_pair_yield_kernel(uint8_t* hashes, const uint64_t* counts, uint32_t n,
                                                            PohBatchScratch* s, uint32_t one, PohYield y) {
    __shared__ uint64_t run_len;
    if (threadIdx.x == 0) pair_yield = y;
    __syncthreads();
    const uint32_t role = threadIdx.x >> 5;
    const bool counted = role == 0 && (threadIdx.x & 31u) == 0;
    const uint32_t place = counted ? poh_place_enter() : 0u;
    pair_persistent<0, true>(hashes, counts, n, s, &run_len, role, 0, 0, one);
    if (counted) poh_place_leave(place);
}

}  // namespace

cudaError_t poh_round_warp_map(const uint32_t** per_slot, const uint32_t** busy_slots) {
    void* a = nullptr;
    void* b = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&a, g_poh_round_warps);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&b, g_poh_busy_slots);
    *per_slot = static_cast<const uint32_t*>(a);
    *busy_slots = static_cast<const uint32_t*>(b);
    return e;
}

// The persistent PoH kernels run for up to seconds beside signature work.
// An SM's split between L1 and shared memory is set for the blocks it holds;
// a block that needs more shared memory than that split gives cannot be
// placed there until the SM drains.  With the driver's own split for these
// kernels (14 KB of shared memory per pair block), the served loop's
// resident signature kernel (60 KB per block) could wait behind running PoH
// launches.  These kernels and that one therefore ask for one split,
// kServeCarveoutPercent of the maximum (sig_service.cu gives the sizes).
cudaError_t preload_poh_batch_kernels() {
    cudaError_t e = load_kernels(poh_hist_kernel, poh_scan_kernel, poh_scatter_kernel, poh_choose_kernel,
                                 poh_requeue_kernel, poh_persistent_kernel<1>, poh_persistent_kernel<4>,
                                 poh_pair_persistent_kernel<1>, poh_pair_persistent_kernel<2>, poh_pair_yield_kernel);
    const int pref = kServeCarveoutPercent;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(poh_persistent_kernel<1>, cudaFuncAttributePreferredSharedMemoryCarveout, pref);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(poh_persistent_kernel<4>, cudaFuncAttributePreferredSharedMemoryCarveout, pref);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(poh_pair_persistent_kernel<1>, cudaFuncAttributePreferredSharedMemoryCarveout, pref);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(poh_pair_persistent_kernel<2>, cudaFuncAttributePreferredSharedMemoryCarveout, pref);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(poh_pair_yield_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pref);
    return e;
}

size_t poh_batch_workspace_size(uint64_t n) { return sizeof(PohBatchScratch) + 4ull * (n ? n : 1); }

cudaError_t launch_poh_pair_direct(uint8_t* hashes, const uint64_t* counts, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (n > 0xffffffe0ull) return cudaErrorInvalidValue;   // 32 * groups must fit 32 bits
    const uint64_t groups = (n + 31) / 32;
    poh_pair_persistent_kernel<1><<<(unsigned)groups, 64, 0, s>>>(hashes, counts, (uint32_t)n, nullptr, 1u);
    return cudaGetLastError();
}

cudaError_t launch_poh_batch(uint8_t* hashes, const uint64_t* counts, uint64_t n, void* workspace,
                             int warps, cudaStream_t s, int form, const PohYield* yield) {
    if (n == 0) return cudaSuccess;
    if (n > 0xffffffffull) return cudaErrorInvalidValue;
    if (form == kPohPairDirect) return launch_poh_pair_direct(hashes, counts, n, s);
    PohBatchScratch* sc = static_cast<PohBatchScratch*>(workspace);
    cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(PohBatchScratch), s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    poh_hist_kernel<<<blocks, 256, 0, s>>>(counts, n, sc, form == kPohAuto);
    poh_scan_kernel<<<1, 32, 0, s>>>(sc);
    poh_scatter_kernel<<<blocks, 256, 0, s>>>(counts, n, sc);
    const uint64_t need = (n + 31) / 32;               // 32-lane groups
    if (form == kPohAuto) {
        // both shapes are enqueued (poh_choose_kernel); the one not chosen
        // finds the queue empty.  Paired: `warps` as given; single: four
        // warps per sub-partition, one per block.
        int dev = 0, sms = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        poh_choose_kernel<<<1, 32, 0, s>>>(sc, (uint32_t)sms, (uint32_t)n);
        const uint64_t pmax = warps / 2 > 0 ? (uint64_t)(warps / 2) : 1;
        const uint64_t pairs = need < pmax ? need : pmax;
        poh_pair_persistent_kernel<1><<<(unsigned)pairs, 64, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
        poh_requeue_kernel<<<1, 32, 0, s>>>(sc);
        const uint64_t smax = 16ull * (uint64_t)sms;
        const uint64_t singles = need < smax ? need : smax;
        poh_persistent_kernel<1><<<(unsigned)singles, 32, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
        return cudaGetLastError();
    }
    const uint64_t wmax = (uint64_t)(warps > 0 ? warps : 1);
    const uint64_t nwarps = need < wmax ? need : wmax;  // single forms: one warp per group
    const uint64_t pmax = wmax / 2 > 0 ? wmax / 2 : 1;  // paired forms: `warps` counts both warps of a pair
    const uint64_t pairs = need < pmax ? need : pmax;
    switch (form) {
        case kPohPackedSingle:
            poh_persistent_kernel<4><<<(unsigned)((nwarps + 3) / 4), 128, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
            break;
        case kPohPair:
            if (yield && yield->chunks && yield->head && yield->tail)
                poh_pair_yield_kernel<<<(unsigned)pairs, 64, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u, *yield);
            else
                poh_pair_persistent_kernel<1><<<(unsigned)pairs, 64, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
            break;
        case kPohPackedPair:
            poh_pair_persistent_kernel<2><<<(unsigned)((pairs + 1) / 2), 128, 0, s>>>(hashes, counts, (uint32_t)n, sc,
                                                                                    1u);
            break;
        default:
            poh_persistent_kernel<1><<<(unsigned)nwarps, 32, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
            break;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Entry point for callers that cannot allocate GPU memory.
//
// Some callers of a PoH verifier are not allowed to call cudaMalloc: a
// validator pipeline whose GPU memory is owned by a pooling allocator with a
// fixed budget, or one that must not take the device-wide synchronisation
// that cudaMalloc / cudaFree can cause in the middle of other streams' work.
// For them the ragged-batch scratch (entry order, bucket counts, queue head)
// lives in this file-scope device array instead of a caller workspace.  The
// array is part of the library image: every GPU that loads the library holds
// it until the process exits.
#include <cstdio>
#include <mutex>

namespace {

constexpr uint64_t kStaticMaxEntries = 262144;   // 1 MiB of entry order + the header

static __device__ __align__(256) uint8_t g_poh_static_scratch[sizeof(PohBatchScratch) + 4 * kStaticMaxEntries];

constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kStaticMaxDevices];   // device address of the array, per device
int g_static_sms[kStaticMaxDevices];

}  // namespace

extern "C" int gb300_poh_verify_batch_static(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems,
                                             void* stream) {
    if (num_elems == 0) return 0;
    if (num_elems > kStaticMaxEntries) {
        fprintf(stderr,
                "gb300_poh_verify_batch_static: %llu entries exceed the static scratch limit of %llu entries\n",
                (unsigned long long)num_elems, (unsigned long long)kStaticMaxEntries);
        return (int)cudaErrorInvalidValue;
    }
    if ((reinterpret_cast<uintptr_t>(hashes) & 15u) || (reinterpret_cast<uintptr_t>(num_hashes) & 7u))
        return (int)cudaErrorMisalignedAddress;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= kStaticMaxDevices) return (int)cudaErrorInvalidDevice;
    void* scratch = nullptr;
    int sms = 0;
    {
        // once per device, with that device current: the array's device
        // address (the host-side symbol is only a stand-in) and the SM count
        std::lock_guard<std::mutex> lk(g_static_mu);
        if (!g_static_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_poh_static_scratch);
            if (e != cudaSuccess) return (int)e;
            int n = 0;
            e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return (int)e;
            e = preload_poh_batch_kernels();           // loaded now, not at a later first launch
            if (e != cudaSuccess) return (int)e;
            g_static_sms[dev] = n > 0 ? n : 1;
            g_static_ptr[dev] = p;
        }
        scratch = g_static_ptr[dev];
        sms = g_static_sms[dev];
    }
    // The array keeps the previous call's contents; launch_poh_batch clears
    // the header (bucket counts, cursors, queue head, shape choice) on every
    // call and rewrites the entry order in full.  Paired warps, one warp per
    // SM sub-partition, unless the counts make single warps faster (chosen
    // on the device; this entry point runs no autotuning, which would
    // allocate).
    return (int)launch_poh_batch(hashes, num_hashes, num_elems, scratch, 4 * sms, static_cast<cudaStream_t>(stream),
                                 kPohAuto);
}
