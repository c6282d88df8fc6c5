// Solana wire-format packets on the device: parse each transaction, expand
// it into the reference's four per-signature arrays and verify, with no host
// pass over the packets.
//
// The reference's ed25519_verify_many (src/cuda-ecc-ed25519/verify.cu:
// 240-258) takes message_lens / public_key_offsets / signature_offsets /
// message_start_offsets computed by its caller, which parses every
// transaction on the host and uploads 16 bytes per signature.  Here the
// packet slots (fixed stride, one data length per packet) go to the GPU as
// they are:
//   1. parse    one thread per packet: signature count (0 = malformed) and
//               the offsets of the signatures, signer keys and message;
//   2. scan     exclusive prefix sum of the counts (per-1024 block scans,
//               one block over the block totals), total on the device;
//   3. expand   one thread per packet writes its signatures' four offsets
//               into the reference's per-signature arrays;
//   4. verify   the persistent signature kernel, its item count read from
//               device memory;
//   5. reduce   one thread per packet: 1 iff it parsed and every one of its
//               signatures verified.
// No step synchronises with the host, so a batch is one stream of launches
// (and one CUDA graph on the host path).
//
// Transaction layout (the published Solana wire format): compact-u16
// signature count n >= 1, n x 64-byte signatures, then the message: an
// optional version byte (top bit set; version 0 only), a 3-byte header
// whose first byte (required signatures) must equal n, a compact-u16
// account-key count k >= n, k x 32-byte keys (the first n sign), and the
// rest.  Signature i verifies with key i over the message bytes up to the
// end of the packet.  compact-u16: 7-bit groups, little-endian, top bit =
// more follow, at most 3 bytes, no redundant zero group, value <= 0xffff.
#include <cuda_runtime.h>
#include "kernels.h"

namespace {

constexpr uint32_t kScanBlock = 1024;

struct PacketWs {
    uint32_t *count, *sig_off, *key_off, *msg_off, *msg_len;   // per packet
    uint32_t *start;                                            // per packet: first signature
    uint32_t *block_sums;                                       // per scan block
    uint32_t *total, *next;                                     // device words
    uint32_t *s_len, *s_key, *s_sig, *s_msg;                    // per signature (capacity)
    uint8_t* s_out;                                             // per signature verdicts
};

uint64_t cap_per_packet(uint64_t stride) {
    const uint64_t c = stride / 64;     // 64 bytes per signature inside the slot
    return c < 0xffff ? c : 0xffff;     // and the compact-u16 limit
}

uint64_t align256(uint64_t x) { return (x + 255) & ~255ull; }

// Carves the workspace; returns its size (ws == nullptr: size only).
uint64_t carve(void* ws, uint32_t n, uint64_t stride, PacketWs* w) {
    const uint64_t cap = (uint64_t)n * cap_per_packet(stride);
    const uint64_t nb = (n + kScanBlock - 1) / kScanBlock;
    uint8_t* base = static_cast<uint8_t*>(ws);
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) -> uint8_t* {
        uint8_t* p = base ? base + off : nullptr;
        off += align256(bytes ? bytes : 1);
        return p;
    };
    PacketWs t;
    t.count = (uint32_t*)take(4ull * n);
    t.sig_off = (uint32_t*)take(4ull * n);
    t.key_off = (uint32_t*)take(4ull * n);
    t.msg_off = (uint32_t*)take(4ull * n);
    t.msg_len = (uint32_t*)take(4ull * n);
    t.start = (uint32_t*)take(4ull * n);
    t.block_sums = (uint32_t*)take(4ull * nb);
    t.total = (uint32_t*)take(8);
    t.next = t.total ? t.total + 1 : nullptr;
    t.s_len = (uint32_t*)take(4ull * cap);
    t.s_key = (uint32_t*)take(4ull * cap);
    t.s_sig = (uint32_t*)take(4ull * cap);
    t.s_msg = (uint32_t*)take(4ull * cap);
    t.s_out = take(cap);
    if (w) *w = t;
    return off;
}

__device__ __forceinline__ bool cu16_read(const uint8_t* p, uint32_t len, uint32_t& pos, uint32_t& val) {
    uint32_t v = 0;
#pragma unroll
    for (uint32_t i = 0; i < 3; i++) {
        if (pos + i >= len) return false;
        const uint32_t b = p[pos + i];
        v |= (b & 0x7fu) << (7 * i);
        if (!(b & 0x80u)) {
            if (i > 0 && b == 0) return false;   // redundant zero group
            if (i == 2 && b > 3) return false;   // above 0xffff
            pos += i + 1;
            val = v;
            return true;
        }
    }
    return false;                                // a fourth byte
}

// Signature count of one transaction (0: malformed); offsets relative to p.
__device__ uint32_t parse_one(const uint8_t* p, uint32_t len, uint32_t& so, uint32_t& ko, uint32_t& mo) {
    uint32_t pos = 0, n = 0, k = 0;
    if (!cu16_read(p, len, pos, n) || n == 0) return 0;
    so = pos;
    if ((uint64_t)pos + 64ull * n > len) return 0;
    pos += 64 * n;
    mo = pos;
    if (pos >= len) return 0;
    uint32_t b = p[pos];
    if (b & 0x80u) {
        if ((b & 0x7fu) != 0) return 0;          // only version 0
        pos++;
    }
    if ((uint64_t)pos + 3 > len) return 0;
    if (p[pos] != n) return 0;                   // required signatures == signatures present
    pos += 3;
    if (!cu16_read(p, len, pos, k) || k < n) return 0;
    ko = pos;
    if ((uint64_t)pos + 32ull * k > len) return 0;
    return n;
}

__global__ void parse_kernel(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, PacketWs w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t base = (uint64_t)i * stride;
    const uint32_t len = lens[i];
    uint32_t so = 0, ko = 0, mo = 0;
    const uint32_t c = len > stride ? 0 : parse_one(data + base, len, so, ko, mo);
    w.count[i] = c;
    w.sig_off[i] = c ? (uint32_t)(base + so) : 0;
    w.key_off[i] = c ? (uint32_t)(base + ko) : 0;
    w.msg_off[i] = c ? (uint32_t)(base + mo) : 0;
    w.msg_len[i] = c ? len - mo : 0;
}

// Exclusive scan of v over a 1024-thread block; returns the block total.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t& excl) {
    __shared__ uint32_t warp_tot[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        warp_tot[lane] = t;                      // inclusive over warps
    }
    __syncthreads();
    excl = x - v + (warp ? warp_tot[warp - 1] : 0);
    const uint32_t total = warp_tot[31];
    __syncthreads();                             // warp_tot reused by the next call
    return total;
}

__global__ void __launch_bounds__(kScanBlock) scan_local_kernel(PacketWs w, uint32_t n) {
    const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
    uint32_t excl;
    const uint32_t tot = block_scan(i < n ? w.count[i] : 0, excl);
    if (i < n) w.start[i] = excl;
    if (threadIdx.x == 0) w.block_sums[blockIdx.x] = tot;
}

// one block: exclusive scan of the block totals, in chunks of 1024
__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(PacketWs w, uint32_t nb) {
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        const uint32_t b = b0 + threadIdx.x;
        uint32_t excl;
        const uint32_t tot = block_scan(b < nb ? w.block_sums[b] : 0, excl);
        if (b < nb) w.block_sums[b] = carry + excl;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        *w.total = carry;
        *w.next = 0;                             // queue head of the verify launch
    }
}

// Per packet: global first signature, then its signatures' four offsets.
__global__ void expand_kernel(PacketWs w, uint32_t n, uint32_t* s_len, uint32_t* s_key, uint32_t* s_sig,
                              uint32_t* s_msg, uint32_t* counts_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s0 = w.start[i] + w.block_sums[i / kScanBlock];
    w.start[i] = s0;
    const uint32_t c = w.count[i];
    if (counts_out) counts_out[i] = c;
    const uint32_t ml = w.msg_len[i], ko = w.key_off[i], so = w.sig_off[i], mo = w.msg_off[i];
    for (uint32_t j = 0; j < c; j++) {
        s_len[s0 + j] = ml;
        s_key[s0 + j] = ko + 32 * j;
        s_sig[s0 + j] = so + 64 * j;
        s_msg[s0 + j] = mo;
    }
}

__global__ void reduce_kernel(PacketWs w, uint32_t n, uint8_t* packet_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = w.count[i], s0 = w.start[i];
    uint32_t ok = c > 0;
    for (uint32_t j = 0; j < c && ok; j++) ok = w.s_out[s0 + j];
    packet_out[i] = ok ? 1 : 0;
}

cudaError_t check_args(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, void* ws,
                       size_t ws_bytes) {
    if (!data || !lens || !ws || stride == 0) return cudaErrorInvalidValue;
    if ((uint64_t)n * stride > 0xffffffffull) return cudaErrorInvalidValue;   // offsets are 32-bit
    if ((uint64_t)n * cap_per_packet(stride) > 0x7fffffffull) return cudaErrorInvalidValue;
    if (ws_bytes < carve(nullptr, n, stride, nullptr)) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(ws) & 255u) || (reinterpret_cast<uintptr_t>(lens) & 3u))
        return cudaErrorMisalignedAddress;
    return cudaSuccess;
}

// Steps 1-3 into the given per-signature arrays.
cudaError_t enqueue_extract(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, const PacketWs& w,
                            uint32_t* s_len, uint32_t* s_key, uint32_t* s_sig, uint32_t* s_msg, uint32_t* counts_out,
                            cudaStream_t s) {
    const uint32_t nb = (n + kScanBlock - 1) / kScanBlock;
    const uint32_t grid = (n + 255) / 256;
    parse_kernel<<<grid, 256, 0, s>>>(data, stride, n, lens, w);
    scan_local_kernel<<<nb, kScanBlock, 0, s>>>(w, n);
    scan_sums_kernel<<<1, kScanBlock, 0, s>>>(w, nb);
    expand_kernel<<<grid, 256, 0, s>>>(w, n, s_len, s_key, s_sig, s_msg, counts_out);
    return cudaGetLastError();
}

}  // namespace

cudaError_t preload_packets_kernels() {
    return load_kernels(parse_kernel, scan_local_kernel, scan_sums_kernel, expand_kernel, reduce_kernel);
}

size_t packets_workspace_size(uint32_t n, uint64_t stride) { return carve(nullptr, n, stride, nullptr); }

uint64_t packets_signature_capacity(uint32_t n, uint64_t stride) { return (uint64_t)n * cap_per_packet(stride); }

cudaError_t launch_packets_extract(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, void* ws,
                                   size_t ws_bytes, uint32_t* message_lens, uint32_t* key_offsets,
                                   uint32_t* sig_offsets, uint32_t* msg_offsets, uint32_t* counts_out,
                                   uint32_t* total_out, cudaStream_t s) {
    if (n == 0) return total_out ? cudaMemsetAsync(total_out, 0, 4, s) : cudaSuccess;
    cudaError_t e = check_args(data, stride, n, lens, ws, ws_bytes);
    if (e != cudaSuccess) return e;
    if (!message_lens || !key_offsets || !sig_offsets || !msg_offsets) return cudaErrorInvalidValue;
    PacketWs w;
    carve(ws, n, stride, &w);
    if ((e = enqueue_extract(data, stride, n, lens, w, message_lens, key_offsets, sig_offsets, msg_offsets,
                             counts_out, s)) != cudaSuccess)
        return e;
    return total_out ? cudaMemcpyAsync(total_out, w.total, 4, cudaMemcpyDeviceToDevice, s) : cudaSuccess;
}

cudaError_t launch_packets_verify(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, void* ws,
                                  size_t ws_bytes, uint8_t* packet_out, uint32_t* counts_out,
                                  const CurveTables* tables, int sig_threads, int sig_blocks_per_sm, int sms,
                                  cudaStream_t s, int verify_window) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = check_args(data, stride, n, lens, ws, ws_bytes);
    if (e != cudaSuccess) return e;
    if (!packet_out) return cudaErrorInvalidValue;
    PacketWs w;
    carve(ws, n, stride, &w);
    if ((e = enqueue_extract(data, stride, n, lens, w, w.s_len, w.s_key, w.s_sig, w.s_msg, counts_out, s)) !=
        cudaSuccess)
        return e;
    const uint64_t cap = packets_signature_capacity(n, stride);
    SigWork sw{};
    sw.v.packets = data;
    sw.v.packets_len = (uint64_t)n * stride;
    sw.v.message_lens = w.s_len;
    sw.v.public_key_offsets = w.s_key;
    sw.v.signature_offsets = w.s_sig;
    sw.v.message_start_offsets = w.s_msg;
    sw.v.n = (uint32_t)cap;                     // capacity; the kernel reads the count
    sw.v.out = w.s_out;
    sw.v.tables = tables;
    sw.v.window = verify_window;
    sw.s = sw.v;
    sw.s.n = 0;
    sw.sign_base = 0xffffffe0u;                 // no sign items
    sw.total_chunks = (uint32_t)((cap + 31) / 32);
    sw.next = w.next;
    sw.count_dev = w.total;
    if ((e = launch_sig_batch(sw, sig_threads, sig_blocks_per_sm, sms, s)) != cudaSuccess) return e;
    reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, n, packet_out);
    return cudaGetLastError();
}
