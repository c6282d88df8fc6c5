// Half-size scalars for Ed25519 verification: for h (mod L) find c, d with
//     c = d h (mod 8L),   d odd and positive,   |c|, d about 2^128.
//
// The reference checks encode([S]B - [h]A) == R (src/cuda-ecc-ed25519/
// verify.cu:137-152, the double-scalar loop of ge.cu:134-171), i.e.
// P = [S]B - [h]A - R is the neutral point.  For such (c, d):
//     [d]P = [dS mod L]B - [c]A - [d]R,
// because B has order L and every curve point has order dividing 8L (so
// [c]A = [dh]A even when A has a small-order component).  The curve group
// has order 8L and d is odd and below L, so [d] is a bijection on it and
// [d]P is neutral exactly when P is: the verdict is unchanged for every
// input.  The variable-base part then needs ~128 doublings instead of ~252.
// (T. Pornin, "Optimized lattice basis reduction in dimension 2, and fast
// Schnorr and EdDSA signature verification", 2020, uses the same identity
// with modulus L; 8L is used here because the reference's check is
// cofactorless.)
//
// (c, d) comes from the half-extended Euclidean algorithm on (8L, h): the
// remainders r_i = t_i h (mod 8L), stopped at the first r below 2^128,
// where |t| <= 8L / r_prev is about 2^128 too (rational reconstruction).
// The remainder sequence is run Lehmer-style: an inner loop of binary steps
// (a <- a - 2^s b) on the top 64 bits of the two remainders, collecting a
// 2x2 matrix of 31-bit cofactors, which one multiply-add then applies to
// the full remainders and cofactors; when the top bits give no step (a
// quotient of 2^32 or more), one exact binary step on the full values.
// Every step is unimodular, so every pair met satisfies r = t h (mod 8L)
// whatever the approximation did; only the length of the result depends on
// it.  The shortest of (r1, t1), (r0, t0), (r0 + r1, t0 + t1),
// (r0 - r1, t0 - t1) with t odd is taken (consecutive t are coprime, so one
// of the first two is odd); if none fits the sizes below, (h, 1) itself,
// which is the full-length check.  So the verdict never depends on the
// reduction, only the time does: h close to a fraction with a small even
// denominator (probability ~2^-120 for a hash) takes the full-length path.
//
// Representation: little-endian 32-bit words; remainders in 9 words and
// cofactors in 6 words, both two's complement rings (intermediate values
// may wrap; every value kept is in range, so the ring arithmetic gives it
// exactly).
#pragma once
#include <stdint.h>

namespace hs {

constexpr int kRem = 9;          // words of a remainder
constexpr int kCof = 6;          // words of a cofactor
constexpr int kMaxOuter = 200;   // a bound only: random h take 4-12 outer steps, h near a small fraction up to ~80

// 8L, little-endian 32-bit words (9th word 0)
__device__ __forceinline__ uint32_t m8L(int i) {
    const uint32_t w[9] = {0xe7ae9f68u, 0xc09318d2u, 0x17bce6b2u, 0xa6f7cef5u, 0u, 0u, 0u, 0x80000000u, 0u};
    return w[i];
}

// r = a + (b ^ m) + (m & 1): a + b when m = 0, a - b when m = ~0
template <int N>
__device__ __forceinline__ void addx(uint32_t* r, const uint32_t* a, const uint32_t* b, uint32_t m) {
    uint32_t c = m & 1u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)a[i] + (b[i] ^ m) + c;
        r[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
}

// r = a << s, 0 <= s <= 31 (in place allowed)
template <int N>
__device__ __forceinline__ void shl(uint32_t* r, const uint32_t* a, uint32_t s) {
#pragma unroll
    for (int i = N - 1; i > 0; i--) r[i] = __funnelshift_l(a[i - 1], a[i], s);
    r[0] = a[0] << s;
}

// r <<= 32 ws words, 0 <= ws < 16 (a four-level select network: register
// arrays are not indexed at run time)
template <int N>
__device__ __forceinline__ void shl_words_var(uint32_t* r, uint32_t ws) {
#pragma unroll
    for (int b = 0; b < 4; b++) {
        const int k = 1 << b;
        if (k >= N) break;
        const bool on = (ws >> b) & 1u;
#pragma unroll
        for (int i = N - 1; i >= 0; i--) r[i] = on ? (i >= k ? r[i - k] : 0u) : r[i];
    }
}

// r = a << s for 0 <= s < 32 N (kWide) or 0 <= s <= 31
template <int N, bool kWide>
__device__ __forceinline__ void shl_any(uint32_t* r, const uint32_t* a, uint32_t s) {
    shl<N>(r, a, s & 31u);
    if (kWide) shl_words_var<N>(r, s >> 5);
}

// all ones when a < b (unsigned)
template <int N>
__device__ __forceinline__ uint32_t lt_mask(const uint32_t* a, const uint32_t* b) {
    uint32_t br = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)a[i] - b[i] - br;
        br = (uint32_t)(t >> 63);
    }
    return 0u - br;
}

// bit length of an unsigned value
template <int N>
__device__ __forceinline__ uint32_t bitlen(const uint32_t* a) {
    uint32_t len = 0;
#pragma unroll
    for (int i = 0; i < N; i++) len = a[i] ? 32u * i + 32u - __clz(a[i]) : len;
    return len;
}

// r = |a| of a signed value; returns all ones when a < 0
template <int N>
__device__ __forceinline__ uint32_t absval(uint32_t* r, const uint32_t* a) {
    const uint32_t m = 0u - (a[N - 1] >> 31);
    uint32_t c = m & 1u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)(a[i] ^ m) + c;
        r[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
    return m;
}

template <int N>
__device__ __forceinline__ void cswap(uint32_t* a, uint32_t* b, uint32_t m) {
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t t = (a[i] ^ b[i]) & m;
        a[i] ^= t;
        b[i] ^= t;
    }
}

// r = a * b (unsigned), NA + NB words
template <int NA, int NB>
__device__ __forceinline__ void mul(uint32_t* r, const uint32_t* a, const uint32_t* b) {
#pragma unroll
    for (int i = 0; i < NA + NB; i++) r[i] = 0;
#pragma unroll
    for (int i = 0; i < NA; i++) {
        uint32_t c = 0;
#pragma unroll
        for (int j = 0; j < NB; j++) {
            const uint64_t t = (uint64_t)a[i] * b[j] + r[i + j] + c;
            r[i + j] = (uint32_t)t;
            c = (uint32_t)(t >> 32);
        }
        r[i + NB] = c;
    }
}

// x >> sh, truncated to 64 bits, for a nonnegative 9-word x
__device__ __forceinline__ uint64_t top64(const uint32_t* x, uint32_t sh) {
    const uint32_t w = sh >> 5, b = sh & 31u;
    uint32_t x0 = 0, x1 = 0, x2 = 0;
#pragma unroll
    for (int k = 0; k < kRem; k++) {
        x0 = (uint32_t)k == w ? x[k] : x0;
        x1 = (uint32_t)k == w + 1 ? x[k] : x1;
        x2 = (uint32_t)k == w + 2 ? x[k] : x2;
    }
    return ((uint64_t)__funnelshift_r(x1, x2, b) << 32) | __funnelshift_r(x0, x1, b);
}

// r = A x + B y in the ring of N words, A and B signed 32-bit (|A|, |B| < 2^31)
template <int N>
__device__ __forceinline__ void lin_comb(uint32_t* r, int32_t A, const uint32_t* x, int32_t B, const uint32_t* y) {
    // the unsigned product by A mod 2^32, minus x << 32 when A < 0
    const uint32_t au = (uint32_t)A, bu = (uint32_t)B;
    const uint32_t ma = 0u - (uint32_t)(A < 0), mb = 0u - (uint32_t)(B < 0);
    uint32_t cx = 0, cy = 0, c = 0, bx = 0, by = 0;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t px = (uint64_t)au * x[i] + cx;
        const uint64_t py = (uint64_t)bu * y[i] + cy;
        cx = (uint32_t)(px >> 32);
        cy = (uint32_t)(py >> 32);
        const uint64_t s = (uint64_t)(uint32_t)px + (uint32_t)py + c;
        c = (uint32_t)(s >> 32);
        // subtract (x << 32) & ma and (y << 32) & mb: word i of each is word i-1
        const uint32_t sx = i ? (x[i - 1] & ma) : 0u, sy = i ? (y[i - 1] & mb) : 0u;
        const uint64_t d1 = (uint64_t)(uint32_t)s - sx - bx;
        bx = (uint32_t)(d1 >> 63);
        const uint64_t d2 = (uint64_t)(uint32_t)d1 - sy - by;
        by = (uint32_t)(d2 >> 63);
        r[i] = (uint32_t)d2;
    }
}

// x = -x in the ring of N words when m is all ones
template <int N>
__device__ __forceinline__ void cneg(uint32_t* x, uint32_t m) {
    uint32_t c = m & 1u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)(x[i] ^ m) + c;
        x[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
}

// Output of the search: |c| (8 words), its sign (all ones when c < 0), d
// (8 words, odd, positive), and the outer steps the reduction ran.
struct HalfScalars {
    uint32_t c[8];
    uint32_t cneg;
    uint32_t d[8];
    uint32_t rounds;
};

// (c, d) for h < L (8 words).  Called by whole warps (the outer loop runs
// until every lane is done).
static __device__ __noinline__ void half_scalars(HalfScalars& o, const uint32_t h[8]) {
    uint32_t r0[kRem], r1[kRem], t0[kCof], t1[kCof];
#pragma unroll
    for (int i = 0; i < kRem; i++) {
        r0[i] = m8L(i);
        r1[i] = i < 8 ? h[i] : 0u;
    }
#pragma unroll
    for (int i = 0; i < kCof; i++) {
        t0[i] = 0;
        t1[i] = i == 0 ? 1u : 0u;
    }
    uint32_t outer = 0;
#pragma unroll 1
    for (;;) {
        const bool active = bitlen<kRem>(r1) > 128u && outer < (uint32_t)kMaxOuter;
        if (!__any_sync(0xffffffffu, active)) break;
        if (!active) continue;
        outer++;
        // inner binary steps on the top 64 bits (r0 >= 2^128 here, so sh >= 65)
        const uint32_t sh = bitlen<kRem>(r0) - 64u;
        uint64_t a = top64(r0, sh), b = top64(r1, sh);
        const uint32_t lim = sh >= 97u ? 32u : 129u - sh;        // stop where r1 would fall below ~2^128
        int64_t A = 1, B = 0, C = 0, D = 1;
        uint32_t n = 0;
#pragma unroll 1
        while (lim < 64u && (b >> lim) != 0) {
            int s = __clzll((long long)b) - __clzll((long long)a);
            if ((b << s) > a) s--;
            if (s >= 32) break;
            const int64_t nA = A - (C << s), nB = B - (D << s);
            if (nA >= (1ll << 31) || nA <= -(1ll << 31) || nB >= (1ll << 31) || nB <= -(1ll << 31)) break;
            a -= b << s;
            A = nA;
            B = nB;
            n++;
            if (a < b) {
                const uint64_t x = a;
                a = b;
                b = x;
                int64_t y = A;
                A = C;
                C = y;
                y = B;
                B = D;
                D = y;
            }
        }
        if (n == 0) {
            // one exact binary step: r0 -= r1 << s, t0 -= t1 << s
            uint32_t s = bitlen<kRem>(r0) - bitlen<kRem>(r1);
            uint32_t x[kRem];
            shl_any<kRem, true>(x, r1, s);
            if (lt_mask<kRem>(r0, x)) {
                s--;
                shl_any<kRem, true>(x, r1, s);
            }
            addx<kRem>(r0, r0, x, ~0u);
            uint32_t y[kCof];
            shl_any<kCof, true>(y, t1, s);
            addx<kCof>(t0, t0, y, ~0u);
        } else {
            uint32_t nr0[kRem], nr1[kRem], nt0[kCof], nt1[kCof];
            lin_comb<kRem>(nr0, (int32_t)A, r0, (int32_t)B, r1);
            lin_comb<kRem>(nr1, (int32_t)C, r0, (int32_t)D, r1);
            lin_comb<kCof>(nt0, (int32_t)A, t0, (int32_t)B, t1);
            lin_comb<kCof>(nt1, (int32_t)C, t0, (int32_t)D, t1);
            const uint32_t m0 = 0u - (nr0[kRem - 1] >> 31), m1 = 0u - (nr1[kRem - 1] >> 31);
            cneg<kRem>(nr0, m0);
            cneg<kCof>(nt0, m0);
            cneg<kRem>(nr1, m1);
            cneg<kCof>(nt1, m1);
#pragma unroll
            for (int i = 0; i < kRem; i++) {
                r0[i] = nr0[i];
                r1[i] = nr1[i];
            }
#pragma unroll
            for (int i = 0; i < kCof; i++) {
                t0[i] = nt0[i];
                t1[i] = nt1[i];
            }
        }
        const uint32_t sw = lt_mask<kRem>(r0, r1);
        cswap<kRem>(r0, r1, sw);
        cswap<kCof>(t0, t1, sw);
    }
    o.rounds = outer;

    // candidates (r1, t1), (r0, t0), (r0 + r1, t0 + t1), (r0 - r1, t0 - t1):
    // the shortest with t odd
    uint32_t pr[kRem], pt[kCof], mr[kRem], mt[kCof];
    addx<kRem>(pr, r0, r1, 0u);
    addx<kCof>(pt, t0, t1, 0u);
    addx<kRem>(mr, r0, r1, ~0u);
    addx<kCof>(mt, t0, t1, ~0u);
    uint32_t best = 0xffffffffu, pick = 4;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t* cr = k == 0 ? r1 : k == 1 ? r0 : k == 2 ? pr : mr;
        const uint32_t* ct = k == 0 ? t1 : k == 1 ? t0 : k == 2 ? pt : mt;
        uint32_t at[kCof];
        absval<kCof>(at, ct);
        const uint32_t lc = bitlen<kRem>(cr), lt = bitlen<kCof>(at);
        const uint32_t l = lc > lt ? lc : lt;
        if ((ct[0] & 1u) && l < best) {
            best = l;
            pick = (uint32_t)k;
        }
    }
    uint32_t cr[kRem], ct[kCof];
#pragma unroll
    for (int i = 0; i < kRem; i++) cr[i] = pick == 0 ? r1[i] : pick == 1 ? r0[i] : pick == 2 ? pr[i] : mr[i];
#pragma unroll
    for (int i = 0; i < kCof; i++) ct[i] = pick == 0 ? t1[i] : pick == 1 ? t0[i] : pick == 2 ? pt[i] : mt[i];
    // d > 0: the pair is negated when t < 0 (-(c, d) satisfies the congruence too)
    const uint32_t tneg = 0u - (ct[kCof - 1] >> 31);
    cneg<kCof>(ct, tneg);
    // sizes of the half-length path: d below 2^160, |c| below 2^253; else
    // (h, 1), the full-length check
    const bool fits = pick < 4 && best <= 252u && bitlen<kCof>(ct) <= 160u;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        o.c[i] = fits ? cr[i] : h[i];
        o.d[i] = fits ? (i < kCof ? ct[i] : 0u) : (i == 0 ? 1u : 0u);
    }
    o.cneg = fits ? tneg : 0u;
}

}  // namespace hs
