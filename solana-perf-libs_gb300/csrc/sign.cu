// Ed25519 batch signing and keypair derivation, one thread per item.
//
// Replaces the reference's ed25519_sign_kernel / ed25519_sign_device
// (src/cuda-ecc-ed25519/sign.cu:9-38, :50-72) and ed25519_create_keypair
// (keypair.cu:6-16).  Deterministic Ed25519:
//   r = SHA-512(sk[32..64) || M) mod L,  R = [r]B,
//   S = (SHA-512(R || A || M) mod L) * sk[0..32) + r  mod L.
// [r]B uses the 64-window comb table (tables.cuh) with a constant-time
// select of each window's entry, as the reference's ge_scalarmult_base does
// (ge.cu:399-500): 64 affine additions, no doublings.
#include <cuda_runtime.h>
#include <atomic>
#include "kernels.h"
#include "tables.cuh"
#include "sha512.cuh"
#include "sc25519.cuh"

#ifndef SIGN_THREADS
#define SIGN_THREADS 128
#endif
#ifndef SIGN_MIN_BLOCKS
#define SIGN_MIN_BLOCKS 0   // 0: no minimum in the launch bounds
#endif
#if SIGN_MIN_BLOCKS > 0
#define SIGN_BOUNDS __launch_bounds__(SIGN_THREADS, SIGN_MIN_BLOCKS)
#else
#define SIGN_BOUNDS __launch_bounds__(SIGN_THREADS)
#endif

namespace {

#include "ed25519_ops.cuh"

// The comb table (48 KB) is staged into shared memory per block: every
// window reads all 8 of its entries, broadcast to the warp, and from global
// memory those reads stalled the kernel on the L1 round trip.
constexpr size_t kCombBytes = sizeof(ge_niels) * COMB_WINDOWS * COMB_ENTRIES;
static_assert(SIGN_THREADS % 32 == 0 && SIGN_THREADS <= 1024, "whole warps");

// One signature in two parts around the block's shared inversion of the
// nonce points' Z (sign_one_tab in ed25519_ops.cuh is the same signature in
// one piece): first r = SHA-512(prefix || M) mod L and R = [r]B in
// projective coordinates, then the encoding of R, the challenge and S.
struct SignWork {
    uint32_t a[8];      // the secret scalar, sk[0..32)
    uint32_t pk[8];
    uint32_t r[8];
    fe X, Y, Z;
    uint64_t mo;
    uint32_t m;
};

// false: an offset is out of range; the signature is zeroed, as the
// one-piece form does
__device__ __forceinline__ bool sign_begin(const SigBatch& a, uint32_t i, const ge_niels* comb, SignWork& w) {
    uint32_t* out = reinterpret_cast<uint32_t*>(a.out + 64ull * i);
    const uint64_t ko = a.signature_offsets[i];   // private key (64 bytes)
    const uint64_t po = a.public_key_offsets[i];
    const uint64_t mo = a.message_start_offsets[i];
    const uint32_t m = a.message_lens[i];
    if (ko + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len) {
#pragma unroll
        for (int k = 0; k < 16; k++) out[k] = 0;
        return false;
    }
    uint32_t sk[16];
#pragma unroll
    for (int k = 0; k < 16; k++) sk[k] = ld_u32_any(a.packets, ko + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) w.pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);
    uint64_t pre[8];
    words_to_be64(pre, sk + 8, 4);
    uint32_t hd[16];
    sha512_prefixed(hd, pre, 4, a.packets, a.packets_len, mo, m);
    sc_reduce512(w.r, hd);
    ge_p3 R;
    scalarmult_base_tab(R, w.r, comb);
    w.X = R.X;
    w.Y = R.Y;
    w.Z = R.Z;
#pragma unroll
    for (int k = 0; k < 8; k++) w.a[k] = sk[k];
    w.mo = mo;
    w.m = m;
    return true;
}

// zi = 1 / Z: R's encoding, h = SHA-512(R || A || M) mod L, S = h a + r mod L
__device__ __forceinline__ void sign_finish(const SigBatch& a, uint32_t i, const SignWork& w, const fe& zi) {
    fe x, y, cx, cy;
    fe_mul(x, w.X, zi);
    fe_mul(y, w.Y, zi);
    fe_canon(cx, x);
    fe_canon(cy, y);
    uint32_t Renc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) Renc[k] = cy.v[k];
    Renc[7] |= (cx.v[0] & 1u) << 31;
    uint64_t pre[8];
    words_to_be64(pre, Renc, 4);
    words_to_be64(pre + 4, w.pk, 4);
    uint32_t hd[16], hram[8], S[8];
    sha512_prefixed(hd, pre, 8, a.packets, a.packets_len, w.mo, w.m);
    sc_reduce512(hram, hd);
    sc_muladd(S, hram, w.a, w.r);
    uint32_t* out = reinterpret_cast<uint32_t*>(a.out + 64ull * i);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        out[k] = Renc[k];
        out[8 + k] = S[k];
    }
}

__device__ __forceinline__ fe fe_shfl_up(const fe& a, uint32_t d) {
    fe r;
#pragma unroll
    for (int k = 0; k < 8; k++) r.v[k] = __shfl_up_sync(0xffffffffu, a.v[k], d);
    return r;
}

__device__ __forceinline__ fe fe_shfl_down(const fe& a, uint32_t d) {
    fe r;
#pragma unroll
    for (int k = 0; k < 8; k++) r.v[k] = __shfl_down_sync(0xffffffffu, a.v[k], d);
    return r;
}

__device__ __forceinline__ void fe_select(fe& r, bool take, const fe& a) {
#pragma unroll
    for (int k = 0; k < 8; k++) r.v[k] = take ? a.v[k] : r.v[k];
}

// 1 / z for every thread of the block (all threads call it; z != 0), with
// one field inversion per block instead of one per thread (Montgomery's
// simultaneous inversion): within each warp, inclusive prefix and suffix
// products of z by shuffles; thread 0 inverts the product of the warps'
// totals and returns each warp the inverse of its own total; then
//   1 / z_i = (z_0 .. z_{i-1}) (z_{i+1} .. z_31) / (z_0 .. z_31).
// An inversion is ~265 field operations: a warp inverting 32 z at once still
// issues all of them, while this costs each warp ~12 multiplications and
// the block one inversion.
__device__ __forceinline__ void block_inverse(fe& zi, const fe& z) {
    constexpr int kWarps = SIGN_THREADS / 32;
    __shared__ fe s_tot[kWarps];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    fe P = z, S = z;   // inclusive prefix and suffix products within the warp
#pragma unroll 1
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const fe up = fe_shfl_up(P, d), dn = fe_shfl_down(S, d);
        fe t;
        fe_mul(t, P, up);
        fe_select(P, lane >= d, t);
        fe_mul(t, S, dn);
        fe_select(S, lane + d < 32u, t);
    }
    fe one;
    fe_set(one, 1);
    fe before = fe_shfl_up(P, 1), after = fe_shfl_down(S, 1);
    fe_select(before, lane == 0, one);
    fe_select(after, lane == 31, one);
    if (lane == 31) s_tot[warp] = P;
    __syncthreads();
    if (threadIdx.x == 0) {
        fe pre[kWarps];
        pre[0] = s_tot[0];
#pragma unroll
        for (int v = 1; v < kWarps; v++) fe_mul(pre[v], pre[v - 1], s_tot[v]);
        fe inv;
        fe_invert(inv, pre[kWarps - 1]);
#pragma unroll
        for (int v = kWarps - 1; v > 0; v--) {
            fe tv;
            fe_mul(tv, inv, pre[v - 1]);   // 1 / T_v
            fe_mul(inv, inv, s_tot[v]);    // 1 / (T_0 .. T_{v-1})
            s_tot[v] = tv;
        }
        s_tot[0] = inv;
    }
    __syncthreads();
    fe t;
    fe_mul(t, before, after);
    fe_mul(zi, t, s_tot[warp]);
}

// SHARED_INV: one inversion per block (block_inverse), for launches of
// several waves; otherwise each thread inverts its own Z (sign_one_tab),
// which uses 128 registers (4 blocks per SM against 3).  Measured on GB300:
// 116,736 signatures in 1.066 against 1.127 ms.
template <bool SHARED_INV>
__global__ void SIGN_BOUNDS ed25519_sign_kernel(SigBatch a) {
    extern __shared__ uint4 s_comb4[];
    const uint4* g = reinterpret_cast<const uint4*>(&a.tables->comb[0][0]);
    for (uint32_t k = threadIdx.x; k < kCombBytes / 16; k += blockDim.x) s_comb4[k] = g[k];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!SHARED_INV) {
        if (i < a.n) sign_one_tab(a, i, reinterpret_cast<const ge_niels*>(s_comb4));
        return;
    }
    // every thread of the block takes part in the shared inversion; one
    // without an item (past n, or offsets out of range) contributes z = 1
    SignWork w;
    const bool live = i < a.n && sign_begin(a, i, reinterpret_cast<const ge_niels*>(s_comb4), w);
    fe z;
    fe_set(z, 1);
    if (live) z = w.Z;
    fe zi;
    block_inverse(zi, z);
    if (live) sign_finish(a, i, w, zi);
}

// seed (32 B) -> sk = SHA-512(seed) with a clamped, pk = [a]B.  The launch
// bound keeps it at 88 registers (5 blocks of 128 per SM); without it the
// compiler took more, and 9,728 keys took 0.500 against 0.369 ms on GB300.
// Sharing one inversion per block, as large signing launches do, gained
// nothing here: 3 blocks per SM instead of 5 cancel the saving (~100 M keys
// per second either way in full waves).
__global__ void __launch_bounds__(SIGN_THREADS) ed25519_keypair_kernel(const uint8_t* seeds, uint8_t* pk_out,
                                                                       uint8_t* sk_out, uint32_t n,
                                                                       const CurveTables* T) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t seed[8];
#pragma unroll
    for (int k = 0; k < 8; k++) seed[k] = ld_u32_any(seeds, 32ull * i + 4 * k, 32ull * n);
    uint64_t pre[4];
    words_to_be64(pre, seed, 4);
    uint32_t hd[16];
    sha512_prefixed(hd, pre, 4, seeds, 32ull * n, 0, 0);
    hd[0] &= ~7u;                                   // sk[0] &= 248
    hd[7] = (hd[7] & 0x3fffffffu) | 0x40000000u;    // sk[31] &= 63; |= 64
    ge_p3 A;
    scalarmult_base(A, hd, T);
    uint32_t enc[8];
    ge_encode_p2(enc, A.X, A.Y, A.Z);
    uint32_t* sk = reinterpret_cast<uint32_t*>(sk_out + 64ull * i);
    uint32_t* pk = reinterpret_cast<uint32_t*>(pk_out + 32ull * i);
#pragma unroll
    for (int k = 0; k < 16; k++) sk[k] = hd[k];
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = enc[k];
}

}  // namespace

namespace {
// The comb (48 KB, dynamic) and the inversion's warp totals (static) exceed
// the 48 KB a block gets without asking; the size is allowed once per
// device, when the kernels are loaded (so never during a graph capture).
cudaError_t sign_shared_opt_in() {
    static std::atomic<uint64_t> opted{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = 1ull << (dev & 63);
    if (opted.load() & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(ed25519_sign_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kCombBytes);
    if (e == cudaSuccess) opted.fetch_or(bit);
    return e;
}

// Signatures from which a launch shares one inversion per block: past one
// full wave of the per-thread form (4 blocks of 128 threads on 152 SMs,
// 77,824).  Below it that form finishes in one wave where the shared form,
// at 3 blocks per SM, needs more: 70,000 signatures took 0.775 against
// 0.770 ms.  In steady state the shared form signs ~8 % more per second.
constexpr uint32_t kSignSharedInvMin = 80000;
}  // namespace

cudaError_t preload_sign_kernels() {
    const cudaError_t e = load_kernels(ed25519_sign_kernel<false>, ed25519_sign_kernel<true>, ed25519_keypair_kernel);
    return e == cudaSuccess ? sign_shared_opt_in() : e;
}

cudaError_t launch_ed25519_sign(const SigBatch& b, cudaStream_t s) {
    if (b.n == 0) return cudaSuccess;
    const unsigned blocks = (b.n + SIGN_THREADS - 1) / SIGN_THREADS;
    if (b.n < kSignSharedInvMin) {
        ed25519_sign_kernel<false><<<blocks, SIGN_THREADS, kCombBytes, s>>>(b);
    } else {
        const cudaError_t e = sign_shared_opt_in();
        if (e != cudaSuccess) return e;
        ed25519_sign_kernel<true><<<blocks, SIGN_THREADS, kCombBytes, s>>>(b);
    }
    return cudaGetLastError();
}

cudaError_t launch_ed25519_keypair(const uint8_t* seeds, uint8_t* pk, uint8_t* sk, uint32_t n,
                                   const CurveTables* tables, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ed25519_keypair_kernel<<<(n + SIGN_THREADS - 1) / SIGN_THREADS, SIGN_THREADS, 0, s>>>(seeds, pk, sk, n, tables);
    return cudaGetLastError();
}
