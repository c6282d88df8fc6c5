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

__global__ void SIGN_BOUNDS ed25519_sign_kernel(SigBatch a) {
    extern __shared__ uint4 s_comb4[];
    const uint4* g = reinterpret_cast<const uint4*>(&a.tables->comb[0][0]);
    for (uint32_t k = threadIdx.x; k < kCombBytes / 16; k += blockDim.x) s_comb4[k] = g[k];
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    sign_one_tab(a, i, reinterpret_cast<const ge_niels*>(s_comb4));
}

// seed (32 B) -> sk = SHA-512(seed) with a clamped, pk = [a]B.
__global__ void ed25519_keypair_kernel(const uint8_t* seeds, uint8_t* pk_out, uint8_t* sk_out, uint32_t n,
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

cudaError_t preload_sign_kernels() { return load_kernels(ed25519_sign_kernel, ed25519_keypair_kernel); }

cudaError_t launch_ed25519_sign(const SigBatch& b, cudaStream_t s) {
    if (b.n == 0) return cudaSuccess;
    ed25519_sign_kernel<<<(b.n + SIGN_THREADS - 1) / SIGN_THREADS, SIGN_THREADS, kCombBytes, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_ed25519_keypair(const uint8_t* seeds, uint8_t* pk, uint8_t* sk, uint32_t n,
                                   const CurveTables* tables, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ed25519_keypair_kernel<<<(n + 127) / 128, 128, 0, s>>>(seeds, pk, sk, n, tables);
    return cudaGetLastError();
}
