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
    uint32_t pad[3];
    uint32_t order[1];          // n entries
};

__device__ __forceinline__ uint32_t bswap_u32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

__device__ __forceinline__ int bucket_of(uint64_t c) { return c ? 64 - __clzll((long long)c) : 0; }

__global__ void poh_hist_kernel(const uint64_t* counts, uint64_t n, PohBatchScratch* s) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&s->hist[bucket_of(counts[i])], 1u);
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

__device__ __forceinline__ void load_entry(const uint8_t* hashes, uint32_t e, uint32_t w[8]) {
    const uint4* p = reinterpret_cast<const uint4*>(hashes + 32ull * e);
    uint4 lo = p[0], hi = p[1];
    w[0] = bswap_u32(lo.x); w[1] = bswap_u32(lo.y); w[2] = bswap_u32(lo.z); w[3] = bswap_u32(lo.w);
    w[4] = bswap_u32(hi.x); w[5] = bswap_u32(hi.y); w[6] = bswap_u32(hi.z); w[7] = bswap_u32(hi.w);
}

__device__ __forceinline__ void store_entry(uint8_t* hashes, uint32_t e, const uint32_t w[8]) {
    uint4* p = reinterpret_cast<uint4*>(hashes + 32ull * e);
    p[0] = make_uint4(bswap_u32(w[0]), bswap_u32(w[1]), bswap_u32(w[2]), bswap_u32(w[3]));
    p[1] = make_uint4(bswap_u32(w[4]), bswap_u32(w[5]), bswap_u32(w[6]), bswap_u32(w[7]));
}

// BW warps per block, each compiled for exactly its block size (a kernel
// bounded for 128 threads but launched with 32 ran 24% slower).
template <int BW>
__global__ void __launch_bounds__(32 * BW) poh_persistent_kernel(uint8_t* hashes, const uint64_t* counts, uint32_t n,
                                                                 PohBatchScratch* s, uint32_t one) {
    const uint32_t lane = threadIdx.x & 31u;
    const PohMul M(one);
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
#pragma unroll 1
            for (uint64_t k = 0; k < r; k++) poh_step_mix<0, 0, 0>(w, M);
            rem -= r;
        }
    }
}

// Paired form: two warps per 32 lanes, as in poh.cu's poh_pair_kernel (warp
// 1 computes the message schedule into shared memory while warp 0 runs the
// rounds), inside the persistent longest-first loop.  Warp 0 owns the queue:
// each refill round it stores finished chains, loads new ones and the step
// count r (the smallest remaining count among its busy lanes), and hands the
// current hash words and r to warp 1 through shared memory at barrier 5;
// then both run r hashes with barriers 1-4 per hash.  r == 0 means every
// lane is done and both warps leave together.
__device__ __forceinline__ uint32_t sched_s0(uint32_t x) { return POH_ROTR(x, 7) ^ POH_ROTR(x, 18) ^ (x >> 3); }
__device__ __forceinline__ uint32_t sched_s1(uint32_t x) { return POH_ROTR(x, 17) ^ POH_ROTR(x, 19) ^ (x >> 10); }

__global__ void __launch_bounds__(64) poh_pair_persistent_kernel(uint8_t* hashes, const uint64_t* counts, uint32_t n,
                                                                 PohBatchScratch* s) {
    __shared__ uint32_t kw[48][32];
    __shared__ uint32_t hout[8][32];
    __shared__ uint64_t run_len;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t iv[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                            0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint64_t rem = 0;
    uint32_t cur = 0xffffffffu;
    bool done = false;
    for (;;) {
        if (warp == 0) {
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
            uint64_t r = done ? ~0ull : rem;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t other = __shfl_xor_sync(0xffffffffu, r, o);
                r = other < r ? other : r;
            }
            if (r == ~0ull) r = 0;
#pragma unroll
            for (int t = 0; t < 8; t++) hout[t][lane] = w[t];
            if (lane == 0) run_len = r;
        }
        asm volatile("bar.sync 5, 64;" ::: "memory");
        const uint64_t r = run_len;
        if (r == 0) break;
        if (warp == 1) {
#pragma unroll
            for (int t = 0; t < 8; t++) w[t] = hout[t][lane];
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
                        const uint32_t x =
                            W[t & 15] + sched_s0(W[(t - 15) & 15]) + W[(t - 7) & 15] + sched_s1(W[(t - 2) & 15]);
                        W[t & 15] = x;
                        kw[t - 16][lane] = x + poh_k(t);
                    }
                    asm volatile("bar.sync %0, 64;" ::"r"(part + 1) : "memory");
                }
                asm volatile("bar.sync 4, 64;" ::: "memory");
#pragma unroll
                for (int t = 0; t < 8; t++) w[t] = hout[t][lane];
            }
        } else {
#pragma unroll 1
            for (uint64_t k = 0; k < r; k++) {
                uint32_t a = iv[0], b = iv[1], c = iv[2], d = iv[3], e = iv[4], f = iv[5], g = iv[6], h = iv[7];
#pragma unroll
                for (int t = 0; t < 64; t++) {
                    if (t == 16 || t == 32 || t == 48) asm volatile("bar.sync %0, 64;" ::"r"(t / 16) : "memory");
                    uint32_t x;
                    if (t < 8) x = w[t] + poh_k(t);
                    else if (t < 16) x = (t == 8 ? 0x80000000u : t == 15 ? 256u : 0u) + poh_k(t);
                    else x = kw[t - 16][lane];
                    const uint32_t t1 =
                        h + (POH_ROTR(e, 6) ^ POH_ROTR(e, 11) ^ POH_ROTR(e, 25)) + ((e & f) ^ (~e & g)) + x;
                    const uint32_t t2 = (POH_ROTR(a, 2) ^ POH_ROTR(a, 13) ^ POH_ROTR(a, 22)) + ((a & b) | (c & (a | b)));
                    h = g;
                    g = f;
                    f = e;
                    e = d + t1;
                    d = c;
                    c = b;
                    b = a;
                    a = t1 + t2;
                }
                if (!done) {
                    w[0] = iv[0] + a; w[1] = iv[1] + b; w[2] = iv[2] + c; w[3] = iv[3] + d;
                    w[4] = iv[4] + e; w[5] = iv[5] + f; w[6] = iv[6] + g; w[7] = iv[7] + h;
                }
#pragma unroll
                for (int t = 0; t < 8; t++) hout[t][lane] = w[t];
                asm volatile("bar.sync 4, 64;" ::: "memory");
            }
            if (!done) rem -= r;
        }
    }
}

}  // namespace

size_t poh_batch_workspace_size(uint64_t n) { return sizeof(PohBatchScratch) + 4ull * (n ? n : 1); }

cudaError_t launch_poh_batch(uint8_t* hashes, const uint64_t* counts, uint64_t n, void* workspace,
                             int warps, cudaStream_t s, int block_warps) {
    if (n == 0) return cudaSuccess;
    if (n > 0xffffffffull) return cudaErrorInvalidValue;
    PohBatchScratch* sc = static_cast<PohBatchScratch*>(workspace);
    cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(PohBatchScratch), s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    poh_hist_kernel<<<blocks, 256, 0, s>>>(counts, n, sc);
    poh_scan_kernel<<<1, 32, 0, s>>>(sc);
    poh_scatter_kernel<<<blocks, 256, 0, s>>>(counts, n, sc);
    // block_warps 1: independent warps spread over as many SMs as possible;
    // 4: independent warps packed one per sub-partition on as few SMs as
    // possible (leaves the rest to other work); 2: paired warps (schedule +
    // rounds) per 32 lanes, poh_pair_persistent_kernel
    if (block_warps != 4 && block_warps != 2) block_warps = 1;
    uint64_t need = (n + 31) / 32;
    uint64_t nwarps = need < (uint64_t)warps ? need : (uint64_t)warps;
    unsigned grid = (unsigned)((nwarps + block_warps - 1) / block_warps);
    if (block_warps == 4) {
        poh_persistent_kernel<4><<<grid, 128, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
    } else if (block_warps == 2) {
        // pairs: `warps` counts both warps of every pair
        const uint64_t pairs_max = (uint64_t)(warps / 2 > 0 ? warps / 2 : 1);
        const unsigned pairs = (unsigned)(need < pairs_max ? need : pairs_max);
        poh_pair_persistent_kernel<<<pairs, 64, 0, s>>>(hashes, counts, (uint32_t)n, sc);
    } else {
        poh_persistent_kernel<1><<<grid, 32, 0, s>>>(hashes, counts, (uint32_t)n, sc, 1u);
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
            g_static_sms[dev] = n > 0 ? n : 1;
            g_static_ptr[dev] = p;
        }
        scratch = g_static_ptr[dev];
        sms = g_static_sms[dev];
    }
    // The array keeps the previous call's contents; launch_poh_batch clears
    // the header (bucket counts, cursors, queue head) on every call and
    // rewrites the entry order in full.  One warp per SM sub-partition, the
    // shape the autotuner picks on GB300.
    return (int)launch_poh_batch(hashes, num_hashes, num_elems, scratch, 4 * sms, static_cast<cudaStream_t>(stream));
}
