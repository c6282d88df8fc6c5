// Per-signature Ed25519 device code shared by the one-call kernels
// (verify.cu, sign.cu) and the persistent batch kernel (sig_batch.cu).
// Included inside an anonymous namespace by each translation unit.
//
// verify_one: reference src/cuda-ecc-ed25519/verify.cu:109-152 (acceptance
// rules restated in verify.cu's header comment).
// sign_one / scalarmult_base: reference sign.cu:9-38, ge.cu:399-500.
#pragma once
#include "kernels.h"
#include "tables.cuh"
#include "sha512.cuh"
#include "sc25519.cuh"


// Carry into each signed radix-16 digit of a scalar < 2^253 (bit i = carry
// into digit i); digit_i = nibble_i + c_i - 16 c_{i+1}, in [-8, 8].
__device__ __forceinline__ uint64_t radix16_carries(const uint32_t h[8]) {
    uint64_t cin = 0;
    uint32_t c = 0;
#pragma unroll
    for (int i = 0; i < 64; i++) {
        cin |= (uint64_t)c << i;
        uint32_t v = ((h[i >> 3] >> ((i & 7) * 4)) & 15u) + c;
        c = v >= 8u;
    }
    return cin;
}

// Same for signed radix-256 digits of S < 2^252, digits in [-128, 128].
__device__ __forceinline__ uint32_t radix256_carries(const uint32_t s[8]) {
    uint32_t cin = 0, c = 0;
#pragma unroll
    for (int k = 0; k < 32; k++) {
        cin |= c << k;
        uint32_t v = ((s[k >> 2] >> ((k & 3) * 8)) & 255u) + c;
        c = v >= 128u;
    }
    return cin;
}

__device__ __forceinline__ void shl_words(uint32_t w[8], int bits) {
#pragma unroll
    for (int i = 7; i > 0; i--) w[i] = __funnelshift_l(w[i - 1], w[i], bits);
    w[0] <<= bits;
}

__device__ __forceinline__ void load_vb(ge_niels& n, const uint32_t* sVB, int e) {
#pragma unroll
    for (int w = 0; w < 8; w++) {
        n.YpX.v[w] = sVB[(0 + w) * VB_ENTRIES + e];
        n.YmX.v[w] = sVB[(8 + w) * VB_ENTRIES + e];
        n.XY2d.v[w] = sVB[(16 + w) * VB_ENTRIES + e];
    }
}

// The signature's 16 words and the public key's 8: read from the packets,
// or taken from `staged` (the same 24 words, staged by the caller).
__device__ __forceinline__ void load_sig_pk(uint32_t sig[16], uint32_t pk[8], const SigBatch& a, uint64_t so,
                                            uint64_t po, const uint32_t* staged) {
    if (staged) {
#pragma unroll
        for (int k = 0; k < 16; k++) sig[k] = staged[k];
#pragma unroll
        for (int k = 0; k < 8; k++) pk[k] = staged[16 + k];
        return;
    }
#pragma unroll
    for (int k = 0; k < 16; k++) sig[k] = ld_u32_any(a.packets, so + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);
}

__device__ bool verify_one(const SigBatch& a, const uint32_t* sVB, uint32_t i, const uint32_t* staged = nullptr) {
    const uint64_t so = a.signature_offsets[i];
    const uint64_t po = a.public_key_offsets[i];
    const uint64_t mo = a.message_start_offsets[i];
    const uint32_t m = a.message_lens[i];
    if (so + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len) return false;

    uint32_t sig[16], pk[8];
    load_sig_pk(sig, pk, a, so, po, staged);

    if (sig[15] & 0xf0000000u) return false;               // S >= 2^252
    if (enc_is_order4(sig) || enc_is_order4(pk)) return false;

    // h = SHA-512(R || A || M) mod L
    uint64_t pre[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        pre[k] = ((uint64_t)bswap32(sig[2 * k]) << 32) | bswap32(sig[2 * k + 1]);
        pre[4 + k] = ((uint64_t)bswap32(pk[2 * k]) << 32) | bswap32(pk[2 * k + 1]);
    }
    uint32_t hd[16], h[8];
    sha512_prefixed(hd, pre, 8, a.packets, a.packets_len, mo, m);
    sc_reduce512(h, hd);

    // -A
    const CurveConsts& K = a.tables->K;
    fe ax, ay;
    if (!ge_decode(ax, ay, pk, K)) return false;
    fe_neg(ax, ax);

    // tab[k] = k * (-A), k = 0..8
    ge_cached tab[9];
    {
        fe d2 = K.d2;
        ge_p3 P1, P2, P3, P4, t3;
        ge_done t;
        P1.X = ax;
        P1.Y = ay;
        fe_set(P1.Z, 1);
        fe_mul(P1.T, ax, ay);
        ge_cached_identity(tab[0]);
        ge_p3_to_cached(tab[1], P1, d2);
        ge_dbl(t, P1.X, P1.Y, P1.Z);
        ge_to_p3(P2, t);
        ge_p3_to_cached(tab[2], P2, d2);
        ge_add_cached(t, P2, tab[1], false);
        ge_to_p3(P3, t);
        ge_p3_to_cached(tab[3], P3, d2);
        ge_dbl(t, P2.X, P2.Y, P2.Z);
        ge_to_p3(P4, t);
        ge_p3_to_cached(tab[4], P4, d2);
        ge_add_cached(t, P4, tab[1], false);
        ge_to_p3(t3, t);
        ge_p3_to_cached(tab[5], t3, d2);
        ge_dbl(t, P3.X, P3.Y, P3.Z);
        ge_to_p3(t3, t);
        ge_p3_to_cached(tab[6], t3, d2);
        ge_add_cached(t, t3, tab[1], false);
        ge_to_p3(t3, t);
        ge_p3_to_cached(tab[7], t3, d2);
        ge_dbl(t, P4.X, P4.Y, P4.Z);
        ge_to_p3(t3, t);
        ge_p3_to_cached(tab[8], t3, d2);
    }

    uint32_t hh[8], ss[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        hh[k] = h[k];
        ss[k] = sig[8 + k];
    }
    const uint64_t hc = radix16_carries(h);
    const uint32_t scar = radix256_carries(ss);

    ge_p3 R;
    ge_p3_identity(R);
#pragma unroll 1
    for (int i = 63; i >= 0; i--) {
        ge_done t;
        if (i != 63) {
            ge_p2 q;
            ge_dbl(t, R.X, R.Y, R.Z);
            ge_to_p2(q, t);
            ge_dbl(t, q.X, q.Y, q.Z);
            ge_to_p2(q, t);
            ge_dbl(t, q.X, q.Y, q.Z);
            ge_to_p2(q, t);
            ge_dbl(t, q.X, q.Y, q.Z);
            ge_to_p3(R, t);
        }
        // digit i of h
        int nib = (int)(hh[7] >> 28);
        shl_words(hh, 4);
        int ci = (int)((hc >> i) & 1u);
        int cn = (i < 63) ? (int)((hc >> (i + 1)) & 1u) : 0;
        int da = nib + ci - 16 * cn;
        int ua = min(da < 0 ? -da : da, 8);      // |digit| <= 8 for h < L; clamp keeps the lookup in the table
        ge_add_cached(t, R, tab[ua], da < 0);
        if ((i & 1) == 0) {
            ge_to_p3(R, t);
            int k = i >> 1;
            int byte = (int)(ss[7] >> 24);
            shl_words(ss, 8);
            int bc = (int)((scar >> k) & 1u);
            int bn = (k < 31) ? (int)((scar >> (k + 1)) & 1u) : 0;
            int db = byte + bc - 256 * bn;
            int ub = min(db < 0 ? -db : db, VB_ENTRIES - 1);
            ge_niels nb;
            load_vb(nb, sVB, ub);
            ge_add_niels(t, R, nb, db < 0);
        }
        ge_p2 q;
        ge_to_p2(q, t);
        R.X = q.X;
        R.Y = q.Y;
        R.Z = q.Z;
    }

    uint32_t enc[8];
    ge_encode_p2(enc, R.X, R.Y, R.Z);
    uint32_t diff = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) diff |= enc[k] ^ sig[k];
    return diff == 0;
}


// W-bit field of h starting at bit pos (h < 2^256, pos + W <= 256).
__device__ __forceinline__ uint32_t bits_at(const uint32_t h[8], int pos, int W) {
    const int w = pos >> 5, o = pos & 31;
    uint32_t v = h[w] >> o;
    if (o + W > 32 && w < 7) v |= h[w + 1] << (32 - o);
    return v & ((1u << W) - 1u);
}

// Carry into each signed radix-2^W digit of h < 2^253 (bit j = carry into
// digit j): digit_j = field_j + c_j - 2^W c_{j+1}, in [-2^(W-1), 2^(W-1)].
template <int W>
__device__ __forceinline__ uint64_t radixw_carries(const uint32_t h[8]) {
    constexpr int NDIG = (253 + W - 1) / W;
    uint64_t cin = 0;
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < NDIG; j++) {
        cin |= (uint64_t)c << j;
        const uint32_t v = bits_at(h, W * j, W) + c;
        c = v >= (1u << (W - 1));
    }
    return cin;
}

// verify_one with a W-bit signed window for h (W = 4 is verify_one's
// fixed-window form).  A Straus loop over bit positions: one doubling per
// bit, the k(-A) addend at multiples of W, the basepoint addend (radix 256,
// shared-memory table) at multiples of 8.  Same verdicts as verify_one.
template <int W>
__device__ bool verify_one_w(const SigBatch& a, const uint32_t* sVB, uint32_t i, const uint32_t* staged = nullptr) {
    constexpr int NDIG = (253 + W - 1) / W;       // digits of h
    constexpr int NTAB = (1 << (W - 1)) + 1;      // k(-A), k = 0..2^(W-1)
    constexpr int TOP = W * (NDIG - 1);
    const uint64_t so = a.signature_offsets[i];
    const uint64_t po = a.public_key_offsets[i];
    const uint64_t mo = a.message_start_offsets[i];
    const uint32_t m = a.message_lens[i];
    if (so + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len) return false;

    uint32_t sig[16], pk[8];
    load_sig_pk(sig, pk, a, so, po, staged);
    if (sig[15] & 0xf0000000u) return false;               // S >= 2^252
    if (enc_is_order4(sig) || enc_is_order4(pk)) return false;

    uint64_t pre[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        pre[k] = ((uint64_t)bswap32(sig[2 * k]) << 32) | bswap32(sig[2 * k + 1]);
        pre[4 + k] = ((uint64_t)bswap32(pk[2 * k]) << 32) | bswap32(pk[2 * k + 1]);
    }
    uint32_t hd[16], h[8];
    sha512_prefixed(hd, pre, 8, a.packets, a.packets_len, mo, m);
    sc_reduce512(h, hd);

    const CurveConsts& K = a.tables->K;
    fe ax, ay;
    if (!ge_decode(ax, ay, pk, K)) return false;
    fe_neg(ax, ax);

    ge_cached tab[NTAB];
    {
        const fe d2 = K.d2;
        ge_p3 P1, Pk;
        ge_done t;
        P1.X = ax;
        P1.Y = ay;
        fe_set(P1.Z, 1);
        fe_mul(P1.T, ax, ay);
        ge_cached_identity(tab[0]);
        ge_p3_to_cached(tab[1], P1, d2);
        ge_dbl(t, P1.X, P1.Y, P1.Z);
        ge_to_p3(Pk, t);
        ge_p3_to_cached(tab[2], Pk, d2);
#pragma unroll 1
        for (int k = 3; k < NTAB; k++) {
            ge_add_cached(t, Pk, tab[1], false);
            ge_to_p3(Pk, t);
            ge_p3_to_cached(tab[k], Pk, d2);
        }
    }

    uint32_t s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = sig[8 + k];
    const uint64_t hc = radixw_carries<W>(h);
    const uint32_t scar = radix256_carries(s);

    ge_p3 R;
    ge_p3_identity(R);
#pragma unroll 1
    for (int pos = TOP; pos >= 0; pos--) {
        const bool addA = (pos % W) == 0, addB = (pos & 7) == 0;
        ge_done t;
        if (pos != TOP) {
            ge_dbl(t, R.X, R.Y, R.Z);
            if (!addA && !addB) {
                ge_p2 q;
                ge_to_p2(q, t);
                R.X = q.X;
                R.Y = q.Y;
                R.Z = q.Z;
                continue;
            }
            ge_to_p3(R, t);
        }
        if (addA) {
            const int j = pos / W;
            const int cj = (int)((hc >> j) & 1u);
            const int cn = (j < NDIG - 1) ? (int)((hc >> (j + 1)) & 1u) : 0;
            const int da = (int)bits_at(h, pos, W) + cj - (cn << W);
            const int ua = min(da < 0 ? -da : da, NTAB - 1);
            ge_add_cached(t, R, tab[ua], da < 0);
            if (addB) ge_to_p3(R, t);
        }
        if (addB) {
            const int k = pos >> 3;
            const int byte = (int)((s[k >> 2] >> ((k & 3) * 8)) & 255u);
            const int bc = (int)((scar >> k) & 1u);
            const int bn = (k < 31) ? (int)((scar >> (k + 1)) & 1u) : 0;
            const int db = byte + bc - 256 * bn;
            const int ub = min(db < 0 ? -db : db, VB_ENTRIES - 1);
            ge_niels nb;
            load_vb(nb, sVB, ub);
            ge_add_niels(t, R, nb, db < 0);
        }
        ge_p2 q;
        ge_to_p2(q, t);
        R.X = q.X;
        R.Y = q.Y;
        R.Z = q.Z;
    }

    uint32_t enc[8];
    ge_encode_p2(enc, R.X, R.Y, R.Z);
    uint32_t diff = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) diff |= enc[k] ^ sig[k];
    return diff == 0;
}

#include "verify_half.cuh"

// Verdict of signature i with window width W of h (4: verify_one, 5:
// verify_one_w<5>), or W = 0: half-size scalars (verify_half.cuh), which
// votes over the warp, so every lane of the warp calls (lanes without a
// signature of their own pass one that exists and drop the verdict).
template <int W>
__device__ __forceinline__ bool verify_window(const SigBatch& a, const uint32_t* sVB, uint32_t i,
                                              const uint32_t* staged = nullptr) {
    if constexpr (W == 0) return verify_half(a, i, staged);
    else if constexpr (W == 4) return verify_one(a, sVB, i, staged);
    else return verify_one_w<W>(a, sVB, i, staged);
}

// [a]B for a < 2^255 (little-endian words), result in extended coordinates.
// comb: the table (j+1) 16^i B as comb[i * COMB_ENTRIES + j], in global or
// shared memory; every entry of a window is read (constant time).
__device__ __forceinline__ void scalarmult_base_tab(ge_p3& R, const uint32_t a[8], const ge_niels* comb) {
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
            const ge_niels& c = comb[i * COMB_ENTRIES + j];
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

__device__ void scalarmult_base(ge_p3& R, const uint32_t a[8], const CurveTables* T) {
    scalarmult_base_tab(R, a, &T->comb[0][0]);
}

__device__ __forceinline__ void sign_one_tab(const SigBatch& a, uint32_t i, const ge_niels* comb) {
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
    scalarmult_base_tab(R, r, comb);
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

__device__ void sign_one(const SigBatch& a, uint32_t i) { sign_one_tab(a, i, &a.tables->comb[0][0]); }

