// Scalars modulo L = 2^252 + 27742317777372353535851937790883648493.
//
// Replaces the reference's sc_reduce (src/cuda-ecc-ed25519/sc.cu:238, a
// 64-byte value mod L in 21-bit limbs) and sc_muladd (sc.cu:565,
// (a*b + c) mod L).  Here: Barrett reduction (Handbook of Applied
// Cryptography, algorithm 14.42, base 2^32, k = 8) of any 512-bit value, with
// mu = floor(2^512 / L).  Both are exact for every input, so the results
// are identical integers.
#pragma once
#include <stdint.h>

// L, little-endian 32-bit words
__device__ __forceinline__ uint32_t sc_L(int i) {
    const uint32_t w[8] = {0x5cf5d3edu, 0x5812631au, 0xa2f79cd6u, 0x14def9deu, 0u, 0u, 0u, 0x10000000u};
    return w[i];
}

// mu = floor(2^512 / L), 260 bits, little-endian 32-bit words
__device__ __forceinline__ uint32_t sc_mu(int i) {
    const uint32_t w[9] = {0x0a2c131bu, 0xed9ce5a3u, 0x086329a7u, 0x2106215du, 0xffffffebu,
                           0xffffffffu, 0xffffffffu, 0xffffffffu, 0x0000000fu};
    return w[i];
}

// r (8 words) = x (16 words, little-endian) mod L
static __device__ __noinline__ void sc_reduce512(uint32_t r[8], const uint32_t x[16]) {
    // q1 = x >> 224 (9 words); q3 = (q1 * mu) >> 288
    uint32_t q1[9];
#pragma unroll
    for (int i = 0; i < 9; i++) q1[i] = x[7 + i];
    uint32_t prod[18];
#pragma unroll
    for (int i = 0; i < 18; i++) prod[i] = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < 9; j++) {
            uint64_t t = (uint64_t)q1[i] * sc_mu(j) + prod[i + j] + carry;
            prod[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        prod[i + 9] = (uint32_t)carry;
    }
    uint32_t q3[9];
#pragma unroll
    for (int i = 0; i < 9; i++) q3[i] = prod[9 + i];
    // r2 = (q3 * L) mod 2^288 ; r = (x mod 2^288) - r2 mod 2^288
    uint32_t r2[9];
#pragma unroll
    for (int i = 0; i < 9; i++) r2[i] = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (i + j < 9) {
                uint64_t t = (uint64_t)q3[i] * sc_L(j) + r2[i + j] + carry;
                r2[i + j] = (uint32_t)t;
                carry = t >> 32;
            }
        }
        if (i + 8 < 9) r2[i + 8] += (uint32_t)carry;
    }
    uint32_t rr[9];
    int64_t borrow = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        int64_t t = (int64_t)x[i] - r2[i] + borrow;
        rr[i] = (uint32_t)t;
        borrow = t >> 32;  // 0 or -1
    }
    // at most two subtractions of L
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
        uint32_t s[9];
        int64_t b = 0;
#pragma unroll
        for (int i = 0; i < 9; i++) {
            int64_t t = (int64_t)rr[i] - (i < 8 ? sc_L(i) : 0u) + b;
            s[i] = (uint32_t)t;
            b = t >> 32;
        }
        bool ge = (b == 0);
#pragma unroll
        for (int i = 0; i < 9; i++) rr[i] = ge ? s[i] : rr[i];
    }
#pragma unroll
    for (int i = 0; i < 8; i++) r[i] = rr[i];
}

// s = (a*b + c) mod L, a, b, c arbitrary 256-bit little-endian values.
static __device__ __noinline__ void sc_muladd(uint32_t s[8], const uint32_t a[8], const uint32_t b[8], const uint32_t c[8]) {
    uint32_t x[16];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = i < 8 ? c[i] : 0u;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            uint64_t t = (uint64_t)a[i] * b[j] + x[i + j] + carry;
            x[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        // propagate into the remaining words (c may have produced carries)
#pragma unroll
        for (int k = i + 8; k < 16; k++) {
            uint64_t t = (uint64_t)x[k] + carry;
            x[k] = (uint32_t)t;
            carry = t >> 32;
        }
    }
    sc_reduce512(s, x);
}
