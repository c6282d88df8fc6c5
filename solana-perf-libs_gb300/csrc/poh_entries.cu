// Solana ledger entries on the GPU: PoH chains with transaction mixins.
//
// The reference's poh_verify_many (src/cuda-poh-verify/poh_verify.cu:80-144)
// only iterates SHA-256.  Its caller, Solana's entry verification, hands it
// each entry's start hash (the previous entry's hash) and hash count, then
// finishes every entry on the host: a transaction entry's last hash mixes in
// the hash of its transactions, and each result is compared with the
// entry's recorded hash.  Here both steps run on the device:
//   entry rule, from the start hash h:
//     no mixin (a tick):  h <- SHA-256(h), num_hashes times;
//     mixin m:            h <- SHA-256(h), max(num_hashes, 1) - 1 times,
//                         then h <- SHA-256(h || m)  (64 bytes, two blocks).
//   * verification: the plain part of every entry runs through the ragged
//     PoH batch (poh_batch.cu: longest first, persistent warps), then one
//     thread per entry applies the mixin and compares;
//   * recording: independent chains, each a sequence of entries, one thread
//     per chain (entries of a chain are serial by definition).
#include <cuda_runtime.h>
#include "kernels.h"
#include "sha256_poh.cuh"

namespace {

__device__ __forceinline__ uint32_t bswap_e(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// One SHA-256 compression of a 16-word (big-endian words) block into st.
__device__ __forceinline__ void sha256_compress(uint32_t st[8], const uint32_t blk[16]) {
    uint32_t W[16];
#pragma unroll
    for (int i = 0; i < 16; i++) W[i] = blk[i];
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
#pragma unroll
    for (int t = 0; t < 64; t++) {
        uint32_t x;
        if (t < 16) {
            x = W[t];
        } else {
            const uint32_t w15 = W[(t - 15) & 15], w2 = W[(t - 2) & 15];
            const uint32_t s0 = POH_ROTR(w15, 7) ^ POH_ROTR(w15, 18) ^ (w15 >> 3);
            const uint32_t s1 = POH_ROTR(w2, 17) ^ POH_ROTR(w2, 19) ^ (w2 >> 10);
            x = W[t & 15] + s0 + W[(t - 7) & 15] + s1;
            W[t & 15] = x;
        }
        const uint32_t S1 = POH_ROTR(e, 6) ^ POH_ROTR(e, 11) ^ POH_ROTR(e, 25);
        const uint32_t S0 = POH_ROTR(a, 2) ^ POH_ROTR(a, 13) ^ POH_ROTR(a, 22);
        const uint32_t t1 = h + S1 + ((e & f) ^ (~e & g)) + poh_k(t) + x;
        const uint32_t t2 = S0 + ((a & b) | (c & (a | b)));
        h = g;
        g = f;
        f = e;
        e = d + t1;
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    st[0] += a; st[1] += b; st[2] += c; st[3] += d;
    st[4] += e; st[5] += f; st[6] += g; st[7] += h;
}

// w <- SHA-256(w || m): the 64-byte message is one block, then a block of
// padding only (0x80, zeros, bit length 512).
__device__ __forceinline__ void mix_step(uint32_t w[8], const uint32_t m[8]) {
    uint32_t st[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                      0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    uint32_t blk[16];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        blk[i] = w[i];
        blk[8 + i] = m[i];
    }
    sha256_compress(st, blk);
#pragma unroll
    for (int i = 0; i < 16; i++) blk[i] = 0;
    blk[0] = 0x80000000u;
    blk[15] = 512u;
    sha256_compress(st, blk);
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = st[i];
}

__device__ __forceinline__ void load_be(uint32_t w[8], const uint8_t* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    const uint4 lo = q[0], hi = q[1];
    w[0] = bswap_e(lo.x); w[1] = bswap_e(lo.y); w[2] = bswap_e(lo.z); w[3] = bswap_e(lo.w);
    w[4] = bswap_e(hi.x); w[5] = bswap_e(hi.y); w[6] = bswap_e(hi.z); w[7] = bswap_e(hi.w);
}

__device__ __forceinline__ void store_be(uint8_t* p, const uint32_t w[8]) {
    uint4* q = reinterpret_cast<uint4*>(p);
    q[0] = make_uint4(bswap_e(w[0]), bswap_e(w[1]), bswap_e(w[2]), bswap_e(w[3]));
    q[1] = make_uint4(bswap_e(w[4]), bswap_e(w[5]), bswap_e(w[6]), bswap_e(w[7]));
}

// The plain part of each entry: start hash copied into the workspace, and
// the count of plain hashes before the mixin (if any).
__global__ void entries_prep_kernel(const uint8_t* start, const uint64_t* num_hashes, const uint8_t* has_mixin,
                                    uint64_t n, uint8_t* ws_hashes, uint64_t* ws_counts) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4* s = reinterpret_cast<const uint4*>(start + 32 * i);
    uint4* d = reinterpret_cast<uint4*>(ws_hashes + 32 * i);
    d[0] = s[0];
    d[1] = s[1];
    const uint64_t c = num_hashes[i];
    ws_counts[i] = has_mixin[i] ? (c ? c - 1 : 0) : c;
}

// The mixin step and the comparison with the recorded hash.
__global__ void entries_finish_kernel(const uint8_t* ws_hashes, const uint8_t* mixins, const uint8_t* has_mixin,
                                      const uint8_t* expected, uint64_t n, uint8_t* ok, uint8_t* out_hashes) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t w[8], x[8];
    load_be(w, ws_hashes + 32 * i);
    if (has_mixin[i]) {
        uint32_t m[8];
        load_be(m, mixins + 32 * i);
        mix_step(w, m);
    }
    load_be(x, expected + 32 * i);
    uint32_t diff = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) diff |= w[k] ^ x[k];
    ok[i] = diff == 0 ? 1 : 0;
    if (out_hashes) store_be(out_hashes + 32 * i, w);
}

// Recording: chain c (one thread) runs entries first[c] .. first[c+1]-1.
// Entries past num_entries are not read (a malformed `first` stops there).
__global__ void __launch_bounds__(32) entries_record_kernel(uint8_t* hashes, uint64_t chains, const uint64_t* first,
                                                            uint64_t num_entries, const uint64_t* num_hashes,
                                                            const uint8_t* mixins, const uint8_t* has_mixin,
                                                            uint8_t* entry_hashes, uint32_t one) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= chains) return;
    uint32_t w[8];
    load_be(w, hashes + 32 * c);
    const PohMul M(one);
    const uint64_t end = first[c + 1] < num_entries ? first[c + 1] : num_entries;
    for (uint64_t e = first[c]; e < end; e++) {
        const bool mix = has_mixin[e] != 0;
        const uint64_t cnt = num_hashes[e];
        const uint64_t plain = mix ? (cnt ? cnt - 1 : 0) : cnt;
#pragma unroll 1
        for (uint64_t k = 0; k < plain; k++) poh_step_mix<0, 0, 0>(w, M);
        if (mix) {
            uint32_t m[8];
            load_be(m, mixins + 32 * e);
            mix_step(w, m);
        }
        store_be(entry_hashes + 32 * e, w);
    }
    store_be(hashes + 32 * c, w);
}

}  // namespace

cudaError_t preload_poh_entries_kernels() {
    return load_kernels(entries_prep_kernel, entries_finish_kernel, entries_record_kernel);
}

size_t poh_entries_workspace_size(uint64_t n) {
    const uint64_t m = n ? n : 1;
    return 32 * m + 8 * m + 256 + poh_batch_workspace_size(m);
}

cudaError_t launch_poh_verify_entries(const uint8_t* start, const uint64_t* num_hashes, const uint8_t* mixins,
                                      const uint8_t* has_mixin, const uint8_t* expected, uint64_t n, uint8_t* ok,
                                      uint8_t* out_hashes, void* ws, int warps, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (n > 0xffffffffull) return cudaErrorInvalidValue;
    uint8_t* wh = static_cast<uint8_t*>(ws);
    uint64_t* wc = reinterpret_cast<uint64_t*>(wh + 32 * n);
    void* wb = wh + ((32 * n + 8 * n + 255) / 256) * 256;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    entries_prep_kernel<<<blocks, 256, 0, s>>>(start, num_hashes, has_mixin, n, wh, wc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = launch_poh_batch(wh, wc, n, wb, warps, s, kPohAuto)) != cudaSuccess) return e;
    entries_finish_kernel<<<blocks, 256, 0, s>>>(wh, mixins, has_mixin, expected, n, ok, out_hashes);
    return cudaGetLastError();
}

cudaError_t launch_poh_record(uint8_t* hashes, uint64_t chains, const uint64_t* first, uint64_t num_entries,
                              const uint64_t* num_hashes, const uint8_t* mixins, const uint8_t* has_mixin,
                              uint8_t* entry_hashes, cudaStream_t s) {
    if (chains == 0) return cudaSuccess;
    const uint64_t blocks = (chains + 31) / 32;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    entries_record_kernel<<<(unsigned)blocks, 32, 0, s>>>(hashes, chains, first, num_entries, num_hashes, mixins,
                                                          has_mixin, entry_hashes, 1u);
    return cudaGetLastError();
}
