// GF(2^255-19) on eight 32-bit limbs for sm_103a.
//
// Replaces the reference's ref10 field code (src/cuda-ecc-ed25519/fe.cu:
// fe_mul :556, fe_sq :982, fe_invert :364, fe_pow22523 :881,
// fe_frombytes :297, fe_tobytes :1386, fe_isnegative / fe_isnonzero).
// Different representation (radix 2^32, values kept in [0, 2^256) and only
// fully reduced when encoded or compared); same residues mod p.
#pragma once
#include <stdint.h>
#include "fe25519_ptx.cuh"

struct fe {
    uint32_t v[8];
};

// Multiply and square are called, not inlined (FE_INLINE_MUL=1 inlines
// them): a verification runs ~3,000 of them from a few dozen call sites, and
// inlining every site made the hot loop tens of KB of code, so warps stalled
// on instruction fetch.  Operands and results stay in registers across the
// call (no stack frame).
#ifndef FE_INLINE_MUL
#define FE_INLINE_MUL 0
#endif
#if FE_INLINE_MUL
__device__ __forceinline__ void fe_mul(fe& r, const fe& a, const fe& b) { fe_mul_wide_ptx(r.v, a.v, b.v); }
__device__ __forceinline__ void fe_sq(fe& r, const fe& a) { fe_sq_ptx(r.v, a.v); }
#else
static __device__ __noinline__ fe fe_mul_call(const fe a, const fe b) {
    fe r;
    fe_mul_wide_ptx(r.v, a.v, b.v);
    return r;
}
static __device__ __noinline__ fe fe_sq_call(const fe a) {
    fe r;
    fe_sq_ptx(r.v, a.v);
    return r;
}
__device__ __forceinline__ void fe_mul(fe& r, const fe& a, const fe& b) { r = fe_mul_call(a, b); }
__device__ __forceinline__ void fe_sq(fe& r, const fe& a) { r = fe_sq_call(a); }
#endif
__device__ __forceinline__ void fe_add(fe& r, const fe& a, const fe& b) { fe_add_ptx(r.v, a.v, b.v); }
__device__ __forceinline__ void fe_sub(fe& r, const fe& a, const fe& b) { fe_sub_ptx(r.v, a.v, b.v); }

__device__ __forceinline__ void fe_set(fe& r, uint32_t x) {
    r.v[0] = x;
#pragma unroll
    for (int i = 1; i < 8; i++) r.v[i] = 0;
}

__device__ __forceinline__ void fe_neg(fe& r, const fe& a) {
    fe z;
    fe_set(z, 0);
    fe_sub(r, z, a);
}

// r = c ? b : a   (branch-free select)
__device__ __forceinline__ void fe_select(fe& r, const fe& a, const fe& b, bool c) {
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = c ? b.v[i] : a.v[i];
}

// a^(2^n) for n >= 1
static __device__ __noinline__ void fe_sqn(fe& r, const fe& a, int n) {
    fe t = a;
#pragma unroll 1
    for (int i = 0; i < n; i++) fe_sq(t, t);
    r = t;
}

// Fully reduced representative in [0, p).
__device__ __forceinline__ void fe_canon(fe& r, const fe& a) {
    uint32_t v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = a.v[i];
    // fold bit 255: x = (x mod 2^255) + 19 * (x >> 255)  (< 2^255 + 19)
    uint32_t top = v[7] >> 31;
    v[7] &= 0x7fffffffu;
    asm("{\n\t"
        ".reg .u32 k;\n\t"
        "mul.lo.u32 k, %8, 19;\n\t"
        "add.cc.u32 %0, %0, k;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.cc.u32 %4, %4, 0;\n\t"
        "addc.cc.u32 %5, %5, 0;\n\t"
        "addc.cc.u32 %6, %6, 0;\n\t"
        "addc.u32 %7, %7, 0;\n\t"
        "}"
        : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7])
        : "r"(top));
    // x >= p  <=>  x + 19 >= 2^255; then x - p = (x + 19) mod 2^255
    uint32_t w[8];
    asm("add.cc.u32 %0, %8, 19;\n\t"
        "addc.cc.u32 %1, %9, 0;\n\t"
        "addc.cc.u32 %2, %10, 0;\n\t"
        "addc.cc.u32 %3, %11, 0;\n\t"
        "addc.cc.u32 %4, %12, 0;\n\t"
        "addc.cc.u32 %5, %13, 0;\n\t"
        "addc.cc.u32 %6, %14, 0;\n\t"
        "addc.u32 %7, %15, 0;\n\t"
        : "=&r"(w[0]), "=&r"(w[1]), "=&r"(w[2]), "=&r"(w[3]), "=&r"(w[4]), "=&r"(w[5]), "=&r"(w[6]), "=&r"(w[7])
        : "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]));
    bool ge_p = (w[7] >> 31) != 0;
    w[7] &= 0x7fffffffu;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = ge_p ? w[i] : v[i];
}

__device__ __forceinline__ bool fe_iszero(const fe& a) {
    fe c;
    fe_canon(c, a);
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) acc |= c.v[i];
    return acc == 0;
}

__device__ __forceinline__ uint32_t fe_isodd(const fe& a) {
    fe c;
    fe_canon(c, a);
    return c.v[0] & 1u;
}

__device__ __forceinline__ bool fe_equal(const fe& a, const fe& b) {
    fe d;
    fe_sub(d, a, b);
    return fe_iszero(d);
}

// Little-endian 32-bit words -> field element, bit 255 ignored, no range
// check (a y >= p simply stands for y mod p, as in the reference decode).
__device__ __forceinline__ void fe_from_words(fe& r, const uint32_t w[8]) {
#pragma unroll
    for (int i = 0; i < 7; i++) r.v[i] = w[i];
    r.v[7] = w[7] & 0x7fffffffu;
}

// z^(2^250 - 1) and z^11: runs of ones z^(2^k - 1) for k = 5, 10, 20, 40,
// 50, 100, 200, 250 (249 squarings, 10 multiplications in total here).
static __device__ __noinline__ void fe_pow2_250_1(fe& out, fe& z11, const fe& z) {
    fe z2, z9, t, e5, e10, e20, e50, e100;
    fe_sq(z2, z);                 // 2
    fe_sqn(t, z2, 2);             // 8
    fe_mul(z9, t, z);             // 9
    fe_mul(z11, z9, z2);          // 11
    fe_sq(t, z11);                // 22
    fe_mul(e5, t, z9);            // 2^5 - 1
    fe_sqn(t, e5, 5);
    fe_mul(e10, t, e5);           // 2^10 - 1
    fe_sqn(t, e10, 10);
    fe_mul(e20, t, e10);          // 2^20 - 1
    fe_sqn(t, e20, 20);
    fe_mul(t, t, e20);            // 2^40 - 1
    fe_sqn(t, t, 10);
    fe_mul(e50, t, e10);          // 2^50 - 1
    fe_sqn(t, e50, 50);
    fe_mul(e100, t, e50);         // 2^100 - 1
    fe_sqn(t, e100, 100);
    fe_mul(t, t, e100);           // 2^200 - 1
    fe_sqn(t, t, 50);
    fe_mul(out, t, e50);          // 2^250 - 1
}

// z^(p-2) = z^(2^255 - 21) = (z^(2^250-1))^(2^5) * z^11
__device__ __forceinline__ void fe_invert(fe& r, const fe& z) {
    fe e250, z11, t;
    fe_pow2_250_1(e250, z11, z);
    fe_sqn(t, e250, 5);
    fe_mul(r, t, z11);
}

// z^((p-5)/8) = z^(2^252 - 3) = (z^(2^250-1))^4 * z
__device__ __forceinline__ void fe_pow22523(fe& r, const fe& z) {
    fe e250, z11, t;
    fe_pow2_250_1(e250, z11, z);
    fe_sqn(t, e250, 2);
    fe_mul(r, t, z);
}
