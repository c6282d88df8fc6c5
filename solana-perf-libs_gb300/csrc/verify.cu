// Ed25519 batch verification, one thread per signature, one fused kernel.
//
// Replaces the reference's three-kernel split (src/cuda-ecc-ed25519/
// verify.cu: ed25519_verify_kernel :207, ed25519_gen_lookup_kernel :193,
// ed25519_scalar_double_kernel :176) which passes h (64 B) and an 8-entry
// table (1280 B) per signature through global memory.  Here everything stays
// on chip except the per-thread 9-entry table of multiples of -A.
//
// Acceptance (bit-exact with the reference, see ge25519.cuh for decoding):
//   1. S = sig[32..64) must have its top nibble clear (verify.cu:60-81: the
//      reduction branch never accepts).
//   2. R (sig[0..32)) and A must not encode a point of order dividing 4
//      (ge.cu:61-82).  R need not be decoded at all: the final check compares
//      against a canonical encoding of a valid point, so an R that does not
//      decode can never match, exactly as when the reference rejects it.
//   3. h = SHA-512(R || A || M) mod L; A must decode (ge.cu:182-222).
//   4. encode([S]B + [h](-A)) == R, byte for byte (verify.cu:137-152).
//
// Scalar multiplication: Horner over 64 signed radix-16 digits of h (table of
// 0..8 times -A per thread) interleaved with 32 signed radix-256 digits of S
// (table of 0..128 times B in shared memory).  Fixed windows keep a warp in
// lock-step: every lane adds at the same iterations (a sliding window, as in
// the reference, makes nearly every iteration an add for some lane).
//
// Batches that leave the GPU idle take a shorter chain per signature: four
// lanes per signature (verify_quad.cuh), or three warps per eight
// signatures with half-size scalars (verify_trio.cuh); the form is picked by
// batch size (launch_ed25519_verify).
#include <cuda_runtime.h>
#include <cstdlib>
#include "kernels.h"
#include "tables.cuh"
#include "sha512.cuh"
#include "sc25519.cuh"

#ifndef VERIFY_THREADS
#define VERIFY_THREADS 128
#endif
#ifndef VERIFY_MIN_BLOCKS
#define VERIFY_MIN_BLOCKS 1
#endif

namespace {

#include "ed25519_ops.cuh"
#include "verify_quad.cuh"
#include "verify_trio.cuh"
#include "verify_half.cuh"

// MINB: blocks per SM the register allocation must allow.  1 lets the
// compiler keep everything in registers (254; 2 blocks of 128 fit); 4 caps
// it at 128 registers, with some spills, for batches large enough to fill
// 4 blocks per SM, where the extra warps hide more latency (measured at
// 116,736 signatures: 4.27 ms against 4.57; at 32,768 it is 4 % slower).
// W: the window width of h (4 or 5), or 0 for half-size scalars
// (verify_half.cuh).  Whole warps run: lanes past the batch repeat its last
// signature and drop the verdict.
template <int W, int MINB>
__global__ void __launch_bounds__(VERIFY_THREADS, MINB) ed25519_verify_kernel(SigBatch a) {
    __shared__ uint32_t sVB[VB_WORDS * VB_ENTRIES];
    if (W != 0) {
        for (int k = threadIdx.x; k < VB_WORDS * VB_ENTRIES; k += blockDim.x) sVB[k] = a.tables->vb[k];
        __syncthreads();
    }
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gi < a.n ? gi : a.n - 1u;
    const bool ok = verify_window<W>(a, sVB, i);
    if (gi < a.n) a.out[gi] = ok ? 1 : 0;
}

// Packet staging for the one-lane kernel: each warp brings the 64-byte
// signatures and 32-byte public keys of its 32 signatures on chip with
// coalesced 16-byte loads and hands each lane its 24 words.
//   * The aligned 16-byte chunks covering a signature (5) and a key (3) are
//     loaded by the whole warp, lane l taking chunk l % 8 of signature
//     4 r + l / 8 in round r (8 rounds), so the 8 lanes of one signature read
//     its 128 bytes together and neighbouring signatures' bytes are
//     neighbours in the packet buffer.
//   * Chunks are written transposed into a per-warp area of shared memory,
//     word k of signature s at raw[k * 33 + s] (structure of arrays; the
//     stride of 33 keeps both the writes and each lane's reads of its own
//     column free of bank conflicts).
//   * Each lane then assembles its signature's and key's words from its
//     column, shifting by the byte offset of the signature within its first
//     chunk (packets need only 4-byte alignment, offsets any).
// A chunk that is not entirely inside the packet buffer is read word by word
// with the same bounds rule as the unstaged path (a word at an offset below
// the buffer length is read), and nothing is read for a signature whose
// fields are out of range (its verdict is false either way).
constexpr int kStageStride = 33;
constexpr int kStageWords = 32 * kStageStride;

__device__ __forceinline__ uint4 stage_chunk(const uint8_t* base, uint64_t len, uintptr_t start) {
    const uintptr_t b0 = reinterpret_cast<uintptr_t>(base);
    if (start >= b0 && start + 16 <= b0 + len) return __ldg(reinterpret_cast<const uint4*>(start));
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uintptr_t at = start + 4u * k;
        w[k] = (at >= b0 && at - b0 < len) ? __ldg(reinterpret_cast<const uint32_t*>(at)) : 0u;
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void stage_sig_pk(uint32_t words[24], const SigBatch& a, uint32_t* raw, uint32_t lane,
                                             uint64_t so, uint64_t po, bool ok) {
    const uintptr_t b0 = reinterpret_cast<uintptr_t>(a.packets);
    const uintptr_t sa = b0 + so, pa = b0 + po;          // this lane's signature and key
    const uint32_t c = lane & 7u;
#pragma unroll 1
    for (uint32_t r = 0; r < 8; r++) {
        const uint32_t src = 4u * r + (lane >> 3);
        const uint64_t s_at = __shfl_sync(0xffffffffu, (unsigned long long)sa, src);
        const uint64_t p_at = __shfl_sync(0xffffffffu, (unsigned long long)pa, src);
        const bool s_ok = __shfl_sync(0xffffffffu, ok ? 1u : 0u, src) != 0u;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (s_ok) {
            const uintptr_t start = c < 5u ? (s_at & ~(uintptr_t)15) + 16u * c : (p_at & ~(uintptr_t)15) + 16u * (c - 5u);
            v = stage_chunk(a.packets, a.packets_len, start);
        }
        raw[(4u * c + 0u) * kStageStride + src] = v.x;
        raw[(4u * c + 1u) * kStageStride + src] = v.y;
        raw[(4u * c + 2u) * kStageStride + src] = v.z;
        raw[(4u * c + 3u) * kStageStride + src] = v.w;
    }
    __syncwarp();
    const uint32_t s_sh = (uint32_t)(sa & 3u) * 8u, s_w = (uint32_t)(sa & 15u) >> 2;
    const uint32_t p_sh = (uint32_t)(pa & 3u) * 8u, p_w = 20u + ((uint32_t)(pa & 15u) >> 2);
#pragma unroll
    for (int k = 0; k < 16; k++)
        words[k] = __funnelshift_r(raw[(s_w + k) * kStageStride + lane], raw[(s_w + k + 1) * kStageStride + lane], s_sh);
#pragma unroll
    for (int k = 0; k < 8; k++)
        words[16 + k] =
            __funnelshift_r(raw[(p_w + k) * kStageStride + lane], raw[(p_w + k + 1) * kStageStride + lane], p_sh);
}

// The one-lane kernel with its signatures and keys staged (above).
template <int W, int MINB>
__global__ void __launch_bounds__(VERIFY_THREADS, MINB) ed25519_verify_staged_kernel(SigBatch a) {
    __shared__ uint32_t sVB[VB_WORDS * VB_ENTRIES];
    __shared__ uint32_t sRaw[VERIFY_THREADS / 32][kStageWords];
    for (int k = threadIdx.x; k < VB_WORDS * VB_ENTRIES; k += blockDim.x) sVB[k] = a.tables->vb[k];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    uint64_t so = 0, po = 0;
    bool ok = false;
    if (i < a.n) {
        so = a.signature_offsets[i];
        po = a.public_key_offsets[i];
        const uint64_t mo = a.message_start_offsets[i];
        const uint32_t m = a.message_lens[i];
        ok = !(so + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len);
    }
    uint32_t words[24];
    stage_sig_pk(words, a, sRaw[threadIdx.x >> 5], lane, so, po, ok);
    if (i >= a.n) return;
    a.out[i] = verify_window<W>(a, sVB, i, words) ? 1 : 0;
}

// Four lanes per signature (verify_quad.cuh): signature t / 4 on lane t % 4.
// A quad leaves the kernel together (blockDim is a multiple of 4).
__global__ void __launch_bounds__(VERIFY_THREADS, VERIFY_MIN_BLOCKS) ed25519_verify_quad_kernel(SigBatch a) {
    __shared__ uint32_t sVB[VB_WORDS * VB_ENTRIES];
    for (int k = threadIdx.x; k < VB_WORDS * VB_ENTRIES; k += blockDim.x) sVB[k] = a.tables->vb[k];
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t >> 2, q = t & 3u;
    if (i >= a.n) return;
    const bool ok = verify_quad(a, sVB, i, q);
    if (q == 0) a.out[i] = ok ? 1 : 0;
}

// Three warps per eight signatures (verify_trio.cuh): warps 3g, 3g + 1,
// 3g + 2 of a block are trio g's verifier, hasher and R worker; signature
// 8 t + l / 4 of trio t on lane l % 4 of each.  Trios past the end of the
// batch repeat its last signature (results dropped), so every warp of
// every trio reaches every barrier.
template <int G>
__global__ void __launch_bounds__(96 * G) ed25519_verify_trio_kernel(SigBatch a) {
    __shared__ TrioShare sh[G];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t trio = warp / 3u, role = warp - 3u * trio;
    const uint64_t gi = ((uint64_t)blockIdx.x * G + trio) * 8u + (lane >> 2);
    const uint32_t i = gi < a.n ? (uint32_t)gi : a.n - 1u;
    const uint32_t bar = 1u + 4u * trio;                     // named barriers bar .. bar + 3 (0 is __syncthreads)
    if (role == 0) {
        const bool ok = trio_verifier(a, sh[trio], i, lane, bar);
        if (gi < a.n && (lane & 3u) == 0) a.out[gi] = ok ? 1 : 0;
    } else if (role == 1) {
        trio_hasher(a, sh[trio], i, lane, bar);
    } else {
        trio_r_worker(a, sh[trio], lane, bar);
    }
}

// The half-size scalars of each h (8 words < L) into out[18 i ..]: |c| (8
// words), c's sign (all ones when negative), d (8 words), the reduction's
// rounds.  Whole warps run (half_scalars votes over the warp); lanes past n
// take h = 0 and write nothing.
__global__ void half_scalars_kernel(const uint32_t* h, uint32_t n, uint32_t* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = i < n ? h[8 * i + k] : 0u;
    hs::HalfScalars r;
    hs::half_scalars(r, x);
    if (i >= n) return;
    uint32_t* o = out + 18 * i;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        o[k] = r.c[k];
        o[9 + k] = r.d[k];
    }
    o[8] = r.cneg;
    o[17] = r.rounds;
}

// 0 = the encoding decodes and is not of order dividing 4.
__global__ void check_small_order_kernel(const uint8_t* pts, uint8_t* out, uint32_t n, const CurveTables* T) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) w[k] = ld_u32_any(pts, 32ull * i + 4 * k, 32ull * n);
    fe x, y;
    bool ok = ge_decode(x, y, w, T->K) && !enc_is_order4(w);
    out[i] = ok ? 0 : 1;
}

}  // namespace

cudaError_t preload_verify_kernels() {
    return load_kernels(ed25519_verify_kernel<4, VERIFY_MIN_BLOCKS>, ed25519_verify_kernel<4, 4>,
                        ed25519_verify_kernel<5, VERIFY_MIN_BLOCKS>, ed25519_verify_quad_kernel,
                        ed25519_verify_trio_kernel<1>, ed25519_verify_trio_kernel<2>, half_scalars_kernel,
                        ed25519_verify_staged_kernel<4, VERIFY_MIN_BLOCKS>, ed25519_verify_staged_kernel<4, 4>,
                        ed25519_verify_kernel<0, VERIFY_MIN_BLOCKS>, ed25519_verify_kernel<0, 4>,
                        check_small_order_kernel);
}

cudaError_t launch_ed25519_verify_form(const SigBatch& b, cudaStream_t s, int form) {
    if (b.n == 0) return cudaSuccess;
    if (form == kVerifyTrio) {
        // one trio per block (its three warps on three sub-partitions of an
        // SM) while that fits the SMs once, else two
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return cudaGetLastError();
        const uint64_t trios = (b.n + 7ull) / 8ull;
        if (trios <= (uint64_t)sms) {
            ed25519_verify_trio_kernel<1><<<(unsigned)trios, 96, 0, s>>>(b);
        } else {
            ed25519_verify_trio_kernel<2><<<(unsigned)((trios + 1) / 2), 192, 0, s>>>(b);
        }
        return cudaGetLastError();
    }
    if (form == kVerifyQuad) {
        const uint64_t threads = 4ull * b.n;
        if (threads > 0xffffffffull) return cudaErrorInvalidValue;
        const uint32_t blocks = (uint32_t)((threads + VERIFY_THREADS - 1) / VERIFY_THREADS);
        ed25519_verify_quad_kernel<<<blocks, VERIFY_THREADS, 0, s>>>(b);
    } else if (form == kVerifyStaged) {
        const uint32_t blocks = (b.n + VERIFY_THREADS - 1) / VERIFY_THREADS;
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return cudaGetLastError();
        if ((uint64_t)b.n >= 4ull * VERIFY_THREADS * (uint64_t)sms)
            ed25519_verify_staged_kernel<4, 4><<<blocks, VERIFY_THREADS, 0, s>>>(b);
        else
            ed25519_verify_staged_kernel<4, VERIFY_MIN_BLOCKS><<<blocks, VERIFY_THREADS, 0, s>>>(b);
    } else {
        const uint32_t blocks = (b.n + VERIFY_THREADS - 1) / VERIFY_THREADS;
        if (b.window == 5) {
            ed25519_verify_kernel<5, VERIFY_MIN_BLOCKS><<<blocks, VERIFY_THREADS, 0, s>>>(b);
        } else {
            int dev = 0, sms = 0;
            if (cudaGetDevice(&dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return cudaGetLastError();
            const bool big = (uint64_t)b.n >= 4ull * VERIFY_THREADS * (uint64_t)sms;
            if (b.window == 0) {
                if (big) ed25519_verify_kernel<0, 4><<<blocks, VERIFY_THREADS, 0, s>>>(b);
                else ed25519_verify_kernel<0, VERIFY_MIN_BLOCKS><<<blocks, VERIFY_THREADS, 0, s>>>(b);
            } else if (big) {
                ed25519_verify_kernel<4, 4><<<blocks, VERIFY_THREADS, 0, s>>>(b);
            } else {
                ed25519_verify_kernel<4, VERIFY_MIN_BLOCKS><<<blocks, VERIFY_THREADS, 0, s>>>(b);
            }
        }
    }
    return cudaGetLastError();
}

// Form by batch size, measured on GB300 (L2 flushed between launches):
//   * three warps per eight signatures up to 40 per SM (6,080): 1,024
//     signatures in 0.28 ms against 0.51 (four lanes) and 1.02 (one lane);
//     4,096 in 0.41 against 0.53; 6,144 in 0.67 against 0.70;
//   * four lanes per signature up to 64 per SM (9,728): 0.72 ms against
//     1.02; break-even with one lane near 12,000 = 78 per SM;
//   * one thread per signature above, where throughput counts: 116,736 in
//     4.6 ms against 8.0 for four lanes.
// GB300_CRYPT_VERIFY_FORM = 0 / 1 / 2 forces one lane / four lanes / three
// warps.
cudaError_t launch_ed25519_verify(const SigBatch& b, cudaStream_t s) {
    static const int forced = getenv("GB300_CRYPT_VERIFY_FORM") ? atoi(getenv("GB300_CRYPT_VERIFY_FORM")) : -1;
    if (forced == kVerifySingle || forced == kVerifyQuad || forced == kVerifyTrio)
        return launch_ed25519_verify_form(b, s, forced);
    static int sms_cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cudaGetLastError();
    int sms = (dev >= 0 && dev < 64) ? __atomic_load_n(&sms_cache[dev], __ATOMIC_RELAXED) : 0;
    if (sms == 0) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return cudaGetLastError();
        if (dev >= 0 && dev < 64) __atomic_store_n(&sms_cache[dev], sms, __ATOMIC_RELAXED);
    }
    const uint64_t n = b.n, m = (uint64_t)sms;
    const int form = n <= 40ull * m ? kVerifyTrio : n <= 64ull * m ? kVerifyQuad : kVerifySingle;
    return launch_ed25519_verify_form(b, s, form);
}

cudaError_t launch_half_scalars(const uint32_t* h, uint32_t n, uint32_t* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    half_scalars_kernel<<<(n + 127) / 128, 128, 0, s>>>(h, n, out);
    return cudaGetLastError();
}

cudaError_t launch_check_small_order(const uint8_t* points, uint8_t* out, uint32_t n, const CurveTables* tables,
                                     cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    check_small_order_kernel<<<(n + 127) / 128, 128, 0, s>>>(points, out, n, tables);
    return cudaGetLastError();
}
