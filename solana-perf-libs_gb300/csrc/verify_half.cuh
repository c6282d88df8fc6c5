// Ed25519 verify, one thread per signature, with half-size scalars: the
// throughput form's chain with ~140 doublings instead of ~252.
//
// Test (half_scalar.cuh gives the argument that it is the reference's
// verdict, src/cuda-ecc-ed25519/verify.cu:137-152, for every input):
//     [S']B + [c](-A) + [d](-R) == neutral point,   S' = d S mod L,
// with c = d h (mod 8L), d odd, |c| and d about 2^128.  Per signature:
//   * SHA-512(R || A || M) mod L, the half-size scalars (c, d), S';
//   * A and R decoded (R canonical and not of order dividing 4, as in the
//     four-lane form), tables of k(-A) and k(-R), k = 0..8;
//   * one Horner loop over the signed radix-16 digits of |c| and d (Straus:
//     the doublings shared), as many digits as the warp's longest scalar;
//   * [S']B from the signing comb (64 additions, no doublings), added at the
//     end; no final inversion (the neutral point is X = 0, Y = Z).
// Against verify_one's ~3,400 field multiplications and squarings per
// signature this is ~2,900: a second decode and table, but about half the
// doublings and no final inversion.
//
// Called by whole warps: the half-size scalar search and the digit count
// vote over the warp, so no lane returns early; a signature that fails a
// check runs to the end on whatever values it has and only its verdict is
// cleared.
#pragma once
#include "half_scalar.cuh"

// tab[k] = k P in cached form, k = 0..8, for P = (x, y) affine (called, not
// inlined: both tables of a signature use the one copy)
static __device__ __noinline__ void half_table(ge_cached tab[9], const fe& x, const fe& y, const fe& d2) {
    ge_p3 P1, P2, P3, P4, t3;
    ge_done t;
    P1.X = x;
    P1.Y = y;
    fe_set(P1.Z, 1);
    fe_mul(P1.T, x, y);
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

// Signed radix-16 digits of x (< 2^253) up to its highest nonzero one.
__device__ __forceinline__ uint32_t half_digits(const uint32_t x[8]) {
    const uint32_t bits = hs::bitlen<8>(x);
    const uint32_t k = (bits + 3u) / 4u;
    return k + (uint32_t)((radix16_carries(x) >> k) & 1u);
}

// Verdict of signature i (every lane of the warp calls; see above).
__device__ bool verify_half(const SigBatch& a, uint32_t i, const uint32_t* staged = nullptr) {
    const uint64_t so0 = a.signature_offsets[i];
    const uint64_t po0 = a.public_key_offsets[i];
    const uint64_t mo0 = a.message_start_offsets[i];
    const uint32_t m0 = a.message_lens[i];
    bool ok = !(so0 + 64 > a.packets_len || po0 + 32 > a.packets_len || mo0 + m0 > a.packets_len);
    const uint64_t so = ok ? so0 : 0, po = ok ? po0 : 0, mo = ok ? mo0 : 0;
    const uint32_t m = ok ? m0 : 0u;                       // read nothing out of range

    uint32_t sig[16], pk[8];
    load_sig_pk(sig, pk, a, so, po, ok ? staged : nullptr);
    ok = ok && !(sig[15] & 0xf0000000u);                   // S >= 2^252
    ok = ok && !enc_is_order4(sig) && !enc_is_order4(pk);
    // R's y >= p: no canonical encoding equals it
    {
        const uint32_t hi_ones = sig[1] & sig[2] & sig[3] & sig[4] & sig[5] & sig[6];
        ok = ok && !((sig[7] & 0x7fffffffu) == 0x7fffffffu && hi_ones == 0xffffffffu && sig[0] >= 0xffffffedu);
    }

    // h = SHA-512(R || A || M) mod L, then (c, d) and S' = d S mod L
    uint64_t pre[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        pre[k] = ((uint64_t)bswap32(sig[2 * k]) << 32) | bswap32(sig[2 * k + 1]);
        pre[4 + k] = ((uint64_t)bswap32(pk[2 * k]) << 32) | bswap32(pk[2 * k + 1]);
    }
    uint32_t digest[16], h[8];
    sha512_prefixed(digest, pre, 8, a.packets, a.packets_len, mo, m);
    sc_reduce512(h, digest);
    hs::HalfScalars hsv;
    hs::half_scalars(hsv, h);
    uint32_t sp[8];
    {
        uint32_t s8[8], prod[16];
#pragma unroll
        for (int k = 0; k < 8; k++) s8[k] = sig[8 + k];
        hs::mul<8, 8>(prod, hsv.d, s8);
        sc_reduce512(sp, prod);
    }
    const uint32_t dc = half_digits(hsv.c), ddg = half_digits(hsv.d);
    const int nd = (int)__reduce_max_sync(0xffffffffu, dc > ddg ? dc : ddg);

    // -A and -R
    const CurveConsts& K = a.tables->K;
    fe ax, ay, rx, ry;
    ok = ge_decode(ax, ay, pk, K) && ok;
    ok = ge_decode(rx, ry, sig, K) && ok;
    fe_neg(ax, ax);
    fe_neg(rx, rx);
    const fe d2 = K.d2;
    ge_cached tA[9], tR[9];
    half_table(tA, ax, ay, d2);
    half_table(tR, rx, ry, d2);

    // [c](-A) + [d](-R), doublings shared
    uint32_t cc[8], dd[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        cc[k] = hsv.c[k];
        dd[k] = hsv.d[k];
    }
    const bool cneg = hsv.cneg != 0;
    const uint64_t hc = radix16_carries(cc), hd = radix16_carries(dd);
    ge_p3 R;
    ge_p3_identity(R);
#pragma unroll 1
    for (int k = 63; k >= 0; k--) {
        const uint32_t nc = cc[7] >> 28, nn = dd[7] >> 28;
        shl_words(cc, 4);
        shl_words(dd, 4);
        if (k >= nd) continue;                             // zero digits above the warp's longest scalar
        ge_done t;
        if (k != nd - 1) {
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
        const int ci = (int)((hc >> k) & 1u), cn = k < 63 ? (int)((hc >> (k + 1)) & 1u) : 0;
        const int ec = (int)nc + ci - 16 * cn;
        const int di = (int)((hd >> k) & 1u), dn = k < 63 ? (int)((hd >> (k + 1)) & 1u) : 0;
        const int ed = (int)nn + di - 16 * dn;
        ge_add_cached(t, R, tA[min(ec < 0 ? -ec : ec, 8)], (ec < 0) != cneg);
        ge_to_p3(R, t);
        ge_add_cached(t, R, tR[min(ed < 0 ? -ed : ed, 8)], ed < 0);
        ge_to_p3(R, t);
    }

    // + [S']B: 64 signed radix-16 digits, window w adding |e_w| 16^w B from
    // the signing comb (the neutral point for a zero digit)
    const ge_niels* comb = &a.tables->comb[0][0];
    const uint64_t sc = radix16_carries(sp);
#pragma unroll 1
    for (int w = 63; w >= 0; w--) {
        const uint32_t nib = sp[7] >> 28;
        shl_words(sp, 4);
        const int ci = (int)((sc >> w) & 1u), cn = w < 63 ? (int)((sc >> (w + 1)) & 1u) : 0;
        const int e = (int)nib + ci - 16 * cn;
        const int u = e < 0 ? -e : e;
        ge_niels n;
        if (u) {
            n = comb[w * COMB_ENTRIES + (u - 1)];
        } else {
            fe_set(n.YpX, 1);
            fe_set(n.YmX, 1);
            fe_set(n.XY2d, 0);
        }
        ge_done t;
        ge_add_niels(t, R, n, e < 0);
        ge_to_p3(R, t);
    }
    return ok && fe_iszero(R.X) && fe_equal(R.Y, R.Z);
}
