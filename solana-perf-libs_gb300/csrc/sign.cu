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

#define SIGN_THREADS 128

namespace {

// [a]B for a < 2^255 (little-endian words), result in extended coordinates.
__device__ void scalarmult_base(ge_p3& R, const uint32_t a[8], const CurveTables* T) {
    // signed radix-16 digits in [-8, 8]
    int8_t e[64];
#pragma unroll
    for (int i = 0; i < 64; i++) e[i] = (int8_t)((a[i >> 3] >> ((i & 7) * 4)) & 15u);
    int carry = 0;
#pragma unroll
    for (int i = 0; i < 63; i++) {
        int v = e[i] + carry;
        carry = (v + 8) >> 4;
        e[i] = (int8_t)(v - (carry << 4));
    }
    e[63] = (int8_t)(e[63] + carry);

    ge_p3_identity(R);
#pragma unroll 1
    for (int i = 0; i < 64; i++) {
        int d = e[i];
        int u = d < 0 ? -d : d;
        ge_niels sel;
        fe_set(sel.YpX, 1);
        fe_set(sel.YmX, 1);
        fe_set(sel.XY2d, 0);
#pragma unroll
        for (int j = 0; j < COMB_ENTRIES; j++) {
            const ge_niels& c = T->comb[i][j];
            bool take = (u == j + 1);
#pragma unroll
            for (int w = 0; w < 8; w++) {
                sel.YpX.v[w] = take ? c.YpX.v[w] : sel.YpX.v[w];
                sel.YmX.v[w] = take ? c.YmX.v[w] : sel.YmX.v[w];
                sel.XY2d.v[w] = take ? c.XY2d.v[w] : sel.XY2d.v[w];
            }
        }
        ge_done t;
        ge_add_niels(t, R, sel, d < 0);
        ge_to_p3(R, t);
    }
}

__device__ __forceinline__ void words_to_be64(uint64_t* out, const uint32_t* w, int nwords64) {
    for (int k = 0; k < nwords64; k++) out[k] = ((uint64_t)bswap32(w[2 * k]) << 32) | bswap32(w[2 * k + 1]);
}

__device__ void sign_one(const SigBatch& a, uint32_t i) {
    uint32_t* out = reinterpret_cast<uint32_t*>(a.out + 64ull * i);
    const uint64_t ko = a.signature_offsets[i];   // private key (64 bytes)
    const uint64_t po = a.public_key_offsets[i];
    const uint64_t mo = a.message_start_offsets[i];
    const uint32_t m = a.message_lens[i];
    if (ko + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len) {
#pragma unroll
        for (int k = 0; k < 16; k++) out[k] = 0;
        return;
    }
    uint32_t sk[16], pk[8];
#pragma unroll
    for (int k = 0; k < 16; k++) sk[k] = ld_u32_any(a.packets, ko + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);

    // r = SHA-512(prefix || M) mod L
    uint64_t pre[8];
    words_to_be64(pre, sk + 8, 4);
    uint32_t hd[16], r[8];
    sha512_prefixed(hd, pre, 4, a.packets, a.packets_len, mo, m);
    sc_reduce512(r, hd);

    ge_p3 R;
    scalarmult_base(R, r, a.tables);
    uint32_t Renc[8];
    ge_encode_p2(Renc, R.X, R.Y, R.Z);

    // hram = SHA-512(R || A || M) mod L ; S = hram * a + r mod L
    words_to_be64(pre, Renc, 4);
    words_to_be64(pre + 4, pk, 4);
    uint32_t hram[8], S[8];
    sha512_prefixed(hd, pre, 8, a.packets, a.packets_len, mo, m);
    sc_reduce512(hram, hd);
    sc_muladd(S, hram, sk, r);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        out[k] = Renc[k];
        out[8 + k] = S[k];
    }
}

__global__ void __launch_bounds__(SIGN_THREADS) ed25519_sign_kernel(SigBatch a) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    sign_one(a, i);
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

cudaError_t launch_ed25519_sign(const SigBatch& b, cudaStream_t s) {
    if (b.n == 0) return cudaSuccess;
    ed25519_sign_kernel<<<(b.n + SIGN_THREADS - 1) / SIGN_THREADS, SIGN_THREADS, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_ed25519_keypair(const uint8_t* seeds, uint8_t* pk, uint8_t* sk, uint32_t n,
                                   const CurveTables* tables, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    ed25519_keypair_kernel<<<(n + 127) / 128, 128, 0, s>>>(seeds, pk, sk, n, tables);
    return cudaGetLastError();
}
