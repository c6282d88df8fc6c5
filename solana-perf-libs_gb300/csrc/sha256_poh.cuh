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

// Rotation on the multiply pipe: for m = 2^(32-n),
//   rotr(x, n) = (x * m mod 2^32) + hi32(x * m)   (the two parts do not overlap)
// = one mul.hi and one mad.lo.  `m` must reach the kernel as a runtime value
// (a kernel argument) or the compiler turns the products back into shifts on
// the ALU pipe, which is the pipe this offloads.
__device__ __forceinline__ uint32_t rotr_mul(uint32_t x, uint32_t m) {
    uint32_t hi, r;
    asm("mul.hi.u32 %0, %1, %2;" : "=r"(hi) : "r"(x), "r"(m));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(m), "r"(hi));
    return r;
}

// Multipliers 2^(32-n) for every SHA-256 rotation, built from a runtime 1.
struct PohMul {
    uint32_t one, r2, r13, r22, r6, r11, r25, r7, r18, r17, r19;
    __device__ explicit PohMul(uint32_t o)
        : one(o), r2(o << 30), r13(one << 19), r22(one << 10), r6(one << 26), r11(one << 21), r25(one << 7),
          r7(one << 25), r18(one << 14), r17(one << 15), r19(one << 13) {}
};

// x + y on the multiply pipe (x * one + y with a runtime one).
__device__ __forceinline__ uint32_t add_mul(uint32_t x, uint32_t y, uint32_t one) {
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x), "r"(one), "r"(y));
    return r;
}

#ifndef POH_ADD_MUL
#define POH_ADD_MUL 0
#endif

// w[0..7]: the 32-byte hash as big-endian words; replaced by SHA-256(w).
// NS0 / NS1 of the three rotations in Sigma0 / Sigma1 of every round, and NSG
// of the two rotations in each schedule sigma, run on the multiply pipe
// (rotr_mul); the rest use funnel shifts on the ALU pipe.  The split
// balances the two pipes of a warp that has its sub-partition to itself.
template <int NS0, int NS1, int NSG>
__device__ __forceinline__ void poh_step_mix(uint32_t w[8], const PohMul& M) {
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
            uint32_t s0 = (NSG >= 1 ? rotr_mul(w15, M.r7) : POH_ROTR(w15, 7)) ^
                          (NSG >= 2 ? rotr_mul(w15, M.r18) : POH_ROTR(w15, 18)) ^ (w15 >> 3);
            uint32_t s1 = (NSG >= 1 ? rotr_mul(w2, M.r17) : POH_ROTR(w2, 17)) ^
                          (NSG >= 2 ? rotr_mul(w2, M.r19) : POH_ROTR(w2, 19)) ^ (w2 >> 10);
            if (POH_ADD_MUL)
                x = add_mul(s1, W[t & 15] + s0 + W[(t - 7) & 15], M.one);
            else
                x = W[t & 15] + s0 + W[(t - 7) & 15] + s1;
            W[t & 15] = x;
        }
        uint32_t S1 = (NS1 >= 1 ? rotr_mul(e, M.r6) : POH_ROTR(e, 6)) ^
                      (NS1 >= 2 ? rotr_mul(e, M.r11) : POH_ROTR(e, 11)) ^
                      (NS1 >= 3 ? rotr_mul(e, M.r25) : POH_ROTR(e, 25));
        uint32_t S0 = (NS0 >= 1 ? rotr_mul(a, M.r2) : POH_ROTR(a, 2)) ^
                      (NS0 >= 2 ? rotr_mul(a, M.r13) : POH_ROTR(a, 13)) ^
                      (NS0 >= 3 ? rotr_mul(a, M.r22) : POH_ROTR(a, 22));
        uint32_t t1 = h + S1 + ((e & f) ^ (~e & g)) + poh_k(t) + x;
        uint32_t t2 = S0 + ((a & b) | (c & (a | b)));
        h = g;
        g = f;
        f = e;
        e = POH_ADD_MUL ? add_mul(d, t1, M.one) : d + t1;
        d = c;
        c = b;
        b = a;
        a = t1 + t2;
    }
    w[0] = iv[0] + a; w[1] = iv[1] + b; w[2] = iv[2] + c; w[3] = iv[3] + d;
    w[4] = iv[4] + e; w[5] = iv[5] + f; w[6] = iv[6] + g; w[7] = iv[7] + h;
}
