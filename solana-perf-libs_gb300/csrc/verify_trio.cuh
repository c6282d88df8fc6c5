// Ed25519 verify with three warps per eight signatures and half-size scalars
// (a "trio"): the latency form for batches that leave the GPU idle.
//
// The four-lane form (verify_quad.cuh) runs one dependent chain per
// signature: SHA-512, the decodes of A and R, then ~252 doublings with the
// [h](-A) and [S]B additions.  Here the test becomes
//     [S']B + [c](-A) + [d](-R) == neutral point,   S' = d S mod L,
// with the half-size scalars (c, d) of half_scalar.cuh (c = d h mod 8L, d
// odd): that is [d]([S]B - [h]A - R) == neutral, i.e. the reference's
// encode([S]B - [h]A) == R (src/cuda-ecc-ed25519/verify.cu:137-152) once R
// is known canonical and decodable (checked as in the four-lane form);
// half_scalar.cuh gives the argument that [d] changes no verdict.  Its
// three independent terms run on three warps of one block, lanes 4k..4k+3
// of each working on signature k of the trio (quad layout of
// verify_quad.cuh):
//   * the verifier decodes A and R (lanes 0-1 / 2-3 of each quad) and hands
//     -R over, builds the table of -A and runs the Horner loop of [c](-A)
//     over ~33 signed radix-16 digits (~130 doublings instead of ~252);
//   * the hasher computes h = SHA-512(R || A || M) mod L, (c, d) and S',
//     hands c and d over, then computes [S']B with the signing comb (64
//     additions, no doublings);
//   * the R worker builds the table of -R and runs the Horner loop of
//     [d](-R) beside the verifier's;
//   * the verifier adds the other two results and tests for the neutral
//     point.
// The warps meet at named barriers (bar.arrive by the producer, bar.sync by
// the consumers), which every warp reaches unconditionally: a rejected or
// padding signature computes on whatever values it has, with its verdict
// cleared, so no warp leaves early.
#pragma once
#include "half_scalar.cuh"

// What the three warps hand each other (shared memory, one per trio),
// signature k of the trio in slot k, lane l's words at [..][l].
struct TrioShare {
    uint32_t c[8][8];          // hasher -> verifier: |c|
    uint32_t d[8][8];          // hasher -> R worker: d (odd, positive)
    uint32_t cneg[8];          // all ones when c < 0
    uint32_t ok[8];            // the hasher's checks: offsets in range, S < 2^252
    uint32_t ndig;             // signed radix-16 digits covering every |c| and d of the trio
    uint32_t r[16][8];         // verifier -> R worker: -R affine (x, y)
    uint32_t q[16][32];        // hasher -> verifier: cached components (c0, c1) of [S']B
    uint32_t dr[16][32];       // R worker -> verifier: cached components of [d](-R)
};

// Barriers of trio g of a block: 1 + 4g .. 4 + 4g (0 is __syncthreads).
enum TrioBarrier : uint32_t { kTrioScalars = 0, kTrioR = 1, kTrioDR = 2, kTrioQ = 3 };

__device__ __forceinline__ void trio_arrive(uint32_t id, uint32_t threads) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
__device__ __forceinline__ void trio_sync(uint32_t id, uint32_t threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// Offsets of signature i with the reference's range rule; false (and all
// zero, so nothing out of range is read) when any field is outside the
// packet buffer.
__device__ __forceinline__ bool trio_offsets(const SigBatch& a, uint32_t i, uint64_t& so, uint64_t& po, uint64_t& mo,
                                             uint32_t& m) {
    so = a.signature_offsets[i];
    po = a.public_key_offsets[i];
    mo = a.message_start_offsets[i];
    m = a.message_lens[i];
    const bool ok = !(so + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len);
    if (!ok) so = po = mo = m = 0;
    return ok;
}

// Signed radix-16 digit i of a scalar given its top nibble (consumed from
// the left) and its carry mask.
__device__ __forceinline__ int trio_digit(uint32_t nib, uint64_t carries, int i) {
    const int ci = (int)((carries >> i) & 1u);
    const int cn = i < 63 ? (int)((carries >> (i + 1)) & 1u) : 0;
    return (int)nib + ci - 16 * cn;
}

// Signed radix-16 digits of x (< 2^253) up to its highest nonzero one.
__device__ __forceinline__ uint32_t trio_digits(const uint32_t x[8]) {
    const uint32_t bits = hs::bitlen<8>(x);
    const uint32_t k = (bits + 3u) / 4u;                     // nibbles
    return k + (uint32_t)((radix16_carries(x) >> k) & 1u);    // and the carry out of the top one
}

// R = [x](table point) by Horner over the nd low signed radix-16 digits of
// x (8 words, consumed), the table holding this lane's cached components of
// k P, k = 0..8; `neg` negates every digit.  R in extended coordinates.
// Called, not inlined, like trio_table: the verifier and the R worker run
// the same code on one SM, so one copy of it serves both from the
// instruction cache.
static __device__ __noinline__ void trio_horner(ge_p3& R, const fe tab[9][2], uint32_t x[8], bool neg, int nd,
                                                const QuadSel& q, uint32_t mask) {
    const uint64_t xc = radix16_carries(x);
    ge_p3_identity(R);
#pragma unroll 1
    for (int k = 63; k >= 0; k--) {
        const uint32_t nib = x[7] >> 28;
        shl_words(x, 4);
        if (k >= nd) continue;                               // zero digits above the trio's longest scalar
        ge_done t;
        if (k != nd - 1) {
            fe X, Y, Z;
            qdbl(t, R.X, R.Y, R.Z, q, mask);
            qto_p2(X, Y, Z, t, q, mask);
            qdbl(t, X, Y, Z, q, mask);
            qto_p2(X, Y, Z, t, q, mask);
            qdbl(t, X, Y, Z, q, mask);
            qto_p2(X, Y, Z, t, q, mask);
            qdbl(t, X, Y, Z, q, mask);
            qto_p3(R, t, q, mask);
        }
        const int e = trio_digit(nib, xc, k);
        const int u = min(e < 0 ? -e : e, 8);
        qadd_cached(t, R, tab[u][0], tab[u][1], (e < 0) != neg, q, mask);
        qto_p3(R, t, q, mask);
    }
}

// quad_table (this lane's components of k P, k = 0..8), called
static __device__ __noinline__ void trio_table(fe tab[9][2], const fe& x, const fe& y, const fe& d2,
                                               const QuadSel& q) {
    quad_table(tab, x, y, d2, q, kQuadAll);
}

// This lane's cached components of P into a hand-over array.
__device__ __forceinline__ void trio_put_cached(uint32_t (*dst)[32], const ge_p3& P, const fe& d2, const QuadSel& q,
                                                uint32_t lane) {
    fe c0, c1;
    qcached_comps(c0, c1, P, d2, q);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        dst[k][lane] = c0.v[k];
        dst[8 + k][lane] = c1.v[k];
    }
}

// p += (the cached point handed over in src)
__device__ __forceinline__ void trio_add_cached(ge_p3& p, const uint32_t (*src)[32], const QuadSel& q, uint32_t lane,
                                                uint32_t mask) {
    fe c0, c1;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        c0.v[k] = src[k][lane];
        c1.v[k] = src[8 + k][lane];
    }
    ge_done t;
    qadd_cached(t, p, c0, c1, false, q, mask);
    qto_p3(p, t, q, mask);
}

// The hasher warp: h, (c, d), S', the hand-over, then [S']B.
__device__ __forceinline__ void trio_hasher(const SigBatch& a, TrioShare& sh, uint32_t i, uint32_t lane,
                                            uint32_t bar) {
    const uint32_t lane_q = lane & 3u, slot = lane >> 2;
    const QuadSel q = quad_sel(lane_q);
    uint64_t so, po, mo;
    uint32_t m;
    bool ok = trio_offsets(a, i, so, po, mo, m);
    uint32_t sig[16], pk[8];
#pragma unroll
    for (int k = 0; k < 16; k++) sig[k] = ld_u32_any(a.packets, so + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);
    ok = ok && !(sig[15] & 0xf0000000u);                    // S >= 2^252

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
    // S' = d S mod L
    uint32_t sp[8];
    {
        uint32_t s8[8], prod[16];
#pragma unroll
        for (int k = 0; k < 8; k++) s8[k] = sig[8 + k];
        hs::mul<8, 8>(prod, hsv.d, s8);
        sc_reduce512(sp, prod);
    }
    const uint32_t dc = trio_digits(hsv.c), dd = trio_digits(hsv.d);
    const uint32_t nd = __reduce_max_sync(0xffffffffu, dc > dd ? dc : dd);
    if (lane_q == 0) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sh.c[slot][k] = hsv.c[k];
            sh.d[slot][k] = hsv.d[k];
        }
        sh.cneg[slot] = hsv.cneg;
        sh.ok[slot] = ok ? 1u : 0u;
    }
    if (lane == 0) sh.ndig = nd > 0u ? nd : 1u;
    trio_arrive(bar + kTrioScalars, 96);

    // [S']B: 64 signed radix-16 digits, window i adding |e_i| 16^i B from the
    // signing comb (the neutral point for a zero digit)
    const uint32_t* comb = reinterpret_cast<const uint32_t*>(&a.tables->comb[0][0]);
    const uint32_t neutral[24] = {1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const uint64_t sc = radix16_carries(sp);
    ge_p3 Q;
    ge_p3_identity(Q);
#pragma unroll 1
    for (int w = 63; w >= 0; w--) {
        const uint32_t nib = sp[7] >> 28;
        shl_words(sp, 4);
        const int e = trio_digit(nib, sc, w);
        const int u = e < 0 ? -e : e;
        const uint32_t* entry = u ? comb + (w * COMB_ENTRIES + (u - 1)) * 24 : neutral;
        ge_done t;
        qadd_niels_at(t, Q, entry, 1, e < 0, q, lane_q, kQuadAll);
        qto_p3(Q, t, q, kQuadAll);
    }
    trio_put_cached(sh.q, Q, a.tables->K.d2, q, lane);
    trio_arrive(bar + kTrioQ, 64);
}

// The R worker: the table of -R (from the verifier's decode) and [d](-R).
__device__ __forceinline__ void trio_r_worker(const SigBatch& a, TrioShare& sh, uint32_t lane, uint32_t bar) {
    const uint32_t lane_q = lane & 3u, slot = lane >> 2;
    const QuadSel q = quad_sel(lane_q);
    trio_sync(bar + kTrioR, 64);
    fe rx, ry;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        rx.v[k] = sh.r[k][slot];
        ry.v[k] = sh.r[8 + k][slot];
    }
    const fe d2 = a.tables->K.d2;
    fe tR[9][2];
    trio_table(tR, rx, ry, d2, q);
    trio_sync(bar + kTrioScalars, 96);
    uint32_t dd[8];
#pragma unroll
    for (int k = 0; k < 8; k++) dd[k] = sh.d[slot][k];
    ge_p3 D;
    trio_horner(D, tR, dd, false, (int)sh.ndig, q, kQuadAll);
    trio_put_cached(sh.dr, D, d2, q, lane);
    trio_arrive(bar + kTrioDR, 64);
}

// The verifier warp; returns the verdict of signature i (every lane).
__device__ __forceinline__ bool trio_verifier(const SigBatch& a, TrioShare& sh, uint32_t i, uint32_t lane,
                                              uint32_t bar) {
    const uint32_t lane_q = lane & 3u, slot = lane >> 2;
    const QuadSel q = quad_sel(lane_q);
    const uint32_t mask = kQuadAll;
    uint64_t so, po, mo;
    uint32_t m;
    bool ok = trio_offsets(a, i, so, po, mo, m);
    uint32_t rw[8], pk[8];
#pragma unroll
    for (int k = 0; k < 8; k++) rw[k] = ld_u32_any(a.packets, so + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);
    ok = ok && !enc_is_order4(rw) && !enc_is_order4(pk);
    ok = ok && enc_y_canonical(rw);                         // R's y >= p: no canonical encoding equals it

    // lanes 0-1 decode A, lanes 2-3 decode R
    const CurveConsts& K = a.tables->K;
    uint32_t enc[8];
    const uint32_t take_pk = 0u - (uint32_t)(lane_q < 2);
#pragma unroll
    for (int k = 0; k < 8; k++) enc[k] = (pk[k] & take_pk) | (rw[k] & ~take_pk);
    fe dx, dy;
    const uint32_t dok = ge_decode(dx, dy, enc, K) ? 1u : 0u;
    const uint32_t okA = __shfl_sync(kQuadAll, dok, 0, 4), okR = __shfl_sync(kQuadAll, dok, 2, 4);
    ok = ok && okA && okR;
    fe ax, ay, rx, ry;
    quad_from(ax, dx, 0, mask);
    quad_from(ay, dy, 0, mask);
    quad_from(rx, dx, 2, mask);
    quad_from(ry, dy, 2, mask);
    fe_neg(rx, rx);                                          // -R, to the R worker
    if (lane_q == 0) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            sh.r[k][slot] = rx.v[k];
            sh.r[8 + k][slot] = ry.v[k];
        }
    }
    trio_arrive(bar + kTrioR, 64);
    fe_neg(ax, ax);                                          // -A
    fe tA[9][2];
    trio_table(tA, ax, ay, K.d2, q);

    trio_sync(bar + kTrioScalars, 96);
    uint32_t cc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) cc[k] = sh.c[slot][k];
    const bool cneg = sh.cneg[slot] != 0;
    ok = ok && sh.ok[slot];
    ge_p3 R;
    trio_horner(R, tA, cc, cneg, (int)sh.ndig, q, mask);

    // + [d](-R) + [S']B, then the neutral-point test: X == 0, Y == Z
    trio_sync(bar + kTrioDR, 64);
    trio_add_cached(R, sh.dr, q, lane, mask);
    trio_sync(bar + kTrioQ, 64);
    trio_add_cached(R, sh.q, q, lane, mask);
    return ok && fe_iszero(R.X) && fe_equal(R.Y, R.Z);
}
