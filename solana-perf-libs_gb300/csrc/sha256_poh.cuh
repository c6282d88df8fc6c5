// One Proof-of-History step: h <- SHA-256(h) for a 32-byte h, in registers.
//
// Replaces the reference's per-step sha256_init / sha256_process /
// sha256_done (src/cuda-sha256/sha256.cu:198-277, called from
// src/cuda-poh-verify/poh_verify.cu:20-25), which round-trips the state and
// a 64-byte buffer through local memory on every step.  A 32-byte message is
// exactly one block whose second half is constant (0x80, zeros, bit length
// 256), so words 8..15 of the schedule are literals; with every round
// unrolled the compiler folds them (and the constant IV feeding round 0)
// into the arithmetic.
#pragma once
#include <stdint.h>

#define POH_ROTR(x, n) __funnelshift_r((x), (x), (n))

__device__ __forceinline__ uint32_t poh_k(int t) {
    const uint32_t K[64] = {
        0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u, 0x923f82a4u, 0xab1c5ed5u,
        0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u, 0x72be5d74u, 0x80deb1feu, 0x9bdc06a7u, 0xc19bf174u,
        0xe49b69c1u, 0xefbe4786u, 0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu, 0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau,
        0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u, 0xc6e00bf3u, 0xd5a79147u, 0x06ca6351u, 0x14292967u,
        0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu, 0x53380d13u, 0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u,
        0xa2bfe8a1u, 0xa81a664bu, 0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u,
        0x19a4c116u, 0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au, 0x5b9cca4fu, 0x682e6ff3u,
        0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u, 0x90befffau, 0xa4506cebu, 0xbef9a3f7u, 0xc67178f2u};
    return K[t];
}

// w[0..7]: the 32-byte hash as big-endian words; replaced by SHA-256(w).
__device__ __forceinline__ void poh_step(uint32_t w[8]) {
    const uint32_t iv[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                            0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
    uint32_t W[16];
#pragma unroll
    for (int i = 0; i < 8; i++) W[i] = w[i];
    W[8] = 0x80000000u;
#pragma unroll
    for (int i = 9; i < 15; i++) W[i] = 0;
    W[15] = 256u;
    uint32_t a = iv[0], b = iv[1], c = iv[2], d = iv[3], e = iv[4], f = iv[5], g = iv[6], h = iv[7];
#pragma unroll
    for (int t = 0; t < 64; t++) {
        uint32_t x;
        if (t < 16) {
            x = W[t];
        } else {
            uint32_t w15 = W[(t - 15) & 15], w2 = W[(t - 2) & 15];
            uint32_t s0 = POH_ROTR(w15, 7) ^ POH_ROTR(w15, 18) ^ (w15 >> 3);
            uint32_t s1 = POH_ROTR(w2, 17) ^ POH_ROTR(w2, 19) ^ (w2 >> 10);
            x = W[t & 15] + s0 + W[(t - 7) & 15] + s1;
            W[t & 15] = x;
        }
        uint32_t t1 = h + (POH_ROTR(e, 6) ^ POH_ROTR(e, 11) ^ POH_ROTR(e, 25)) + ((e & f) ^ (~e & g)) + poh_k(t) + x;
        uint32_t t2 = (POH_ROTR(a, 2) ^ POH_ROTR(a, 13) ^ POH_ROTR(a, 22)) + ((a & b) | (c & (a | b)));
        h = g;
        g = f;
        f = e;
        e = d + t1;
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    w[0] = iv[0] + a; w[1] = iv[1] + b; w[2] = iv[2] + c; w[3] = iv[3] + d;
    w[4] = iv[4] + e; w[5] = iv[5] + f; w[6] = iv[6] + g; w[7] = iv[7] + h;
}
