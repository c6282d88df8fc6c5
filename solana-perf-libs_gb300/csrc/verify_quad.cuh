// Ed25519 verify with four lanes per signature (a "quad": lanes 4k..4k+3).
//
// One thread per signature is latency-bound on small batches: a verification
// is a chain of ~3,000 dependent field operations (about 1 ms on one warp).
// Each Edwards doubling and addition, however, is two stages of four
// independent multiplications (dbl-2008-hwcd: X^2, Y^2, Z^2, (X+Y)^2, then
// EF, GH, FG, EH; unified addition: (Y1-X1)(Y2-X2), (Y1+X1)(Y2+X2), T1 2dT2,
// Z1 2Z2, then the same four products).  Here lane q of the quad computes
// product q of every stage and the quad exchanges the four results with
// width-4 shuffles, so the [h](-A) + [S]B loop runs one multiplication per
// stage instead of four.
//
// Serial parts are shared out where the code is the same for every lane:
//   * lanes 0-1 decode A while lanes 2-3 decode R (same instructions,
//     different words);
//   * the reference's final step, encode([S]B + [h](-A)) == R bytes
//     (src/cuda-ecc-ed25519/verify.cu:137-152), becomes a projective
//     comparison with the decoded R: X == x_R Z and Y == y_R Z.  The two
//     agree: an encoding is canonical, so R must have y < p (checked
//     explicitly) and a y on the curve (R decodes); given y, the sign bit
//     fixes x because x_R != 0 (x = 0 means y = +-1, which the small-order
//     test has already rejected).  This removes the final inversion.
// SHA-512 and the decode chains run on all four lanes of a quad.  The
// verdicts are those of verify_one for every input.
//
// Every lane of the warp reaches every shuffle: a rejected signature keeps
// computing (on whatever values it has) and only its verdict is cleared, so
// the shuffles name the whole warp.  A mask of the quad alone made each
// shuffle a warp-synchronising branch, and lane-indexed operand choices are
// bit masks, not conditionals, so that the four lanes never diverge around a
// multiplication.
#pragma once

constexpr uint32_t kQuadAll = 0xffffffffu;

// per-lane selection masks: lo = all ones on lanes 1 and 3 of the quad,
// hi = all ones on lanes 2 and 3, m3 = all ones on lane 3
struct QuadSel {
    uint32_t lo, hi, m3;
};
__device__ __forceinline__ QuadSel quad_sel(uint32_t q) {
    QuadSel s;
    s.lo = 0u - (q & 1u);
    s.hi = 0u - ((q >> 1) & 1u);
    s.m3 = s.lo & s.hi;
    return s;
}

// msk ? b : a per bit (one three-input logic op)
__device__ __forceinline__ uint32_t bsel(uint32_t a, uint32_t b, uint32_t msk) { return (b & msk) | (a & ~msk); }

__device__ __forceinline__ void quad_gather4(const fe& m, fe& o0, fe& o1, fe& o2, fe& o3, uint32_t mask) {
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t v = m.v[w];
        o0.v[w] = __shfl_sync(kQuadAll, v, 0, 4);
        o1.v[w] = __shfl_sync(kQuadAll, v, 1, 4);
        o2.v[w] = __shfl_sync(kQuadAll, v, 2, 4);
        o3.v[w] = __shfl_sync(kQuadAll, v, 3, 4);
    }
}

__device__ __forceinline__ void quad_gather3(const fe& m, fe& o0, fe& o1, fe& o2, uint32_t mask) {
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t v = m.v[w];
        o0.v[w] = __shfl_sync(kQuadAll, v, 0, 4);
        o1.v[w] = __shfl_sync(kQuadAll, v, 1, 4);
        o2.v[w] = __shfl_sync(kQuadAll, v, 2, 4);
    }
}

__device__ __forceinline__ void quad_from(fe& r, const fe& m, int src, uint32_t mask) {
#pragma unroll
    for (int w = 0; w < 8; w++) r.v[w] = __shfl_sync(kQuadAll, m.v[w], src, 4);
}

// r = msk ? b : a, branch-free (msk all ones or zero)
__device__ __forceinline__ void fe_select_m(fe& r, const fe& a, const fe& b, uint32_t msk) {
#pragma unroll
    for (int w = 0; w < 8; w++) r.v[w] = (b.v[w] & msk) | (a.v[w] & ~msk);
}

// r = (a0, a1, a2, a3)[q], branch-free: a two-level select tree
__device__ __forceinline__ void fe_pick4(fe& r, const fe& a0, const fe& a1, const fe& a2, const fe& a3,
                                         const QuadSel& q) {
#pragma unroll
    for (int w = 0; w < 8; w++) r.v[w] = bsel(bsel(a0.v[w], a1.v[w], q.lo), bsel(a2.v[w], a3.v[w], q.lo), q.hi);
}

// Doubling, first stage (four squarings), all lanes get (E, F, G, H).
__device__ __forceinline__ void qdbl(ge_done& r, const fe& X, const fe& Y, const fe& Z, const QuadSel& q, uint32_t mask) {
    fe s, op, m, a, b, c, ss;
    fe_add(s, X, Y);
    fe_pick4(op, X, Y, Z, s, q);
    fe_sq(m, op);
    quad_gather4(m, a, b, c, ss, mask);
    fe_add(c, c, c);
    fe_add(r.H, a, b);
    fe_sub(r.E, ss, r.H);
    fe_sub(r.G, b, a);
    fe_sub(r.F, c, r.G);
}

// Second stage: X = EF, Y = GH, Z = FG (and T = EH).
__device__ __forceinline__ void qto_p3(ge_p3& R, const ge_done& c, const QuadSel& q, uint32_t mask) {
    fe o1, o2, m;
    fe_pick4(o1, c.E, c.G, c.F, c.E, q);
    fe_pick4(o2, c.F, c.H, c.G, c.H, q);
    fe_mul(m, o1, o2);
    quad_gather4(m, R.X, R.Y, R.Z, R.T, mask);
}

__device__ __forceinline__ void qto_p2(fe& X, fe& Y, fe& Z, const ge_done& c, const QuadSel& q, uint32_t mask) {
    fe o1, o2, m;
    fe_pick4(o1, c.E, c.G, c.F, c.E, q);
    fe_pick4(o2, c.F, c.H, c.G, c.H, q);
    fe_mul(m, o1, o2);
    quad_gather3(m, X, Y, Z, mask);
}

// Shared tail of the additions: products a, b, c, d -> (E, F, G, H).
__device__ __forceinline__ void qadd_finish(ge_done& r, const fe& m, bool neg, uint32_t mask) {
    fe a, b, c, d, f, g;
    quad_gather4(m, a, b, c, d, mask);
    fe_sub(r.E, b, a);
    fe_add(r.H, b, a);
    fe_sub(f, d, c);
    fe_add(g, d, c);
    const uint32_t nm = 0u - (uint32_t)neg;
    fe_select_m(r.F, f, g, nm);
    fe_select_m(r.G, g, f, nm);
}

// p +- k(-A): the lane's own components of the cached entry, (c0, c1) =
// lane 0 (Y-X, Y+X), lane 1 (Y+X, Y-X), lane 2 (2dT, 2dT), lane 3 (2Z, 2Z);
// the operand is c1 when subtracting, c0 when adding.
__device__ __forceinline__ void qadd_cached(ge_done& r, const ge_p3& p, const fe& c0, const fe& c1, bool neg,
                                            const QuadSel& q, uint32_t mask) {
    fe ypx, ymx, o1, o2, m;
    fe_add(ypx, p.Y, p.X);
    fe_sub(ymx, p.Y, p.X);
    fe_pick4(o1, ymx, ypx, p.T, p.Z, q);
    fe_select_m(o2, c0, c1, 0u - (uint32_t)neg);
    fe_mul(m, o1, o2);
    qadd_finish(r, m, neg, mask);
}

// p +- n for an affine point n in niels form (y+x, y-x, 2dxy), word k of
// component j at n[(8 j + k) * stride]: lane 0 reads y-x (y+x when
// subtracting), lane 1 y+x (y-x), lane 2 2dxy, lane 3 multiplies Z by 2
// (the affine addend has Z = 1).
__device__ __forceinline__ void qadd_niels_at(ge_done& r, const ge_p3& p, const uint32_t* n, int stride, bool neg,
                                              const QuadSel& q, uint32_t lane_q, uint32_t mask) {
    fe ypx, ymx, o1, o2, m;
    fe_add(ypx, p.Y, p.X);
    fe_sub(ymx, p.Y, p.X);
    fe_pick4(o1, ymx, ypx, p.T, p.Z, q);
    // component read: lane 0 y-x (y+x when subtracting), lane 1 the other,
    // lanes 2-3 2dxy (lane 3's operand is replaced by 2 below)
    const uint32_t flip = (uint32_t)neg ^ (lane_q & 1u);
    const int comp = lane_q >= 2 ? 2 : (int)(flip ^ 1u);          // 0 y+x, 1 y-x, 2 2dxy
    const uint32_t two0 = 2u & q.m3;
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t v = n[(comp * 8 + w) * stride];
        o2.v[w] = (v & ~q.m3) | (w == 0 ? two0 : 0u);
    }
    fe_mul(m, o1, o2);
    qadd_finish(r, m, neg, mask);
}

// p +- (entry e of the basepoint table in shared memory, word-major)
__device__ __forceinline__ void qadd_niels(ge_done& r, const ge_p3& p, const uint32_t* sVB, int e, bool neg,
                                           const QuadSel& q, uint32_t lane_q, uint32_t mask) {
    qadd_niels_at(r, p, sVB + e, VB_ENTRIES, neg, q, lane_q, mask);
}

// This lane's two components of the cached form of P.
__device__ __forceinline__ void qcached_comps(fe& c0, fe& c1, const ge_p3& P, const fe& d2, const QuadSel& q) {
    fe ypx, ymx, z2, t2d;
    fe_add(ypx, P.Y, P.X);
    fe_sub(ymx, P.Y, P.X);
    fe_add(z2, P.Z, P.Z);
    fe_mul(t2d, P.T, d2);
    fe_pick4(c0, ymx, ypx, t2d, z2, q);
    fe_pick4(c1, ypx, ymx, t2d, z2, q);
}

// This lane's components of k P for k = 0..8, P = (x, y) affine: entry k
// holds (c0, c1) of the cached form (see qadd_cached).
__device__ __forceinline__ void quad_table(fe tq[9][2], const fe& x, const fe& y, const fe& d2, const QuadSel& q,
                                           uint32_t mask) {
    ge_p3 P1, P2, P3, P4, t3;
    ge_done t;
    P1.X = x;
    P1.Y = y;
    fe_set(P1.Z, 1);
    fe_mul(P1.T, x, y);
    {
        fe one, two, zero;
        fe_set(one, 1);
        fe_set(two, 2);
        fe_set(zero, 0);
        fe_pick4(tq[0][0], one, one, zero, two, q);
        tq[0][1] = tq[0][0];
    }
    qcached_comps(tq[1][0], tq[1][1], P1, d2, q);
    qdbl(t, P1.X, P1.Y, P1.Z, q, mask);
    qto_p3(P2, t, q, mask);
    qcached_comps(tq[2][0], tq[2][1], P2, d2, q);
    qadd_cached(t, P2, tq[1][0], tq[1][1], false, q, mask);
    qto_p3(P3, t, q, mask);
    qcached_comps(tq[3][0], tq[3][1], P3, d2, q);
    qdbl(t, P2.X, P2.Y, P2.Z, q, mask);
    qto_p3(P4, t, q, mask);
    qcached_comps(tq[4][0], tq[4][1], P4, d2, q);
    qadd_cached(t, P4, tq[1][0], tq[1][1], false, q, mask);
    qto_p3(t3, t, q, mask);
    qcached_comps(tq[5][0], tq[5][1], t3, d2, q);
    qdbl(t, P3.X, P3.Y, P3.Z, q, mask);
    qto_p3(t3, t, q, mask);
    qcached_comps(tq[6][0], tq[6][1], t3, d2, q);
    qadd_cached(t, t3, tq[1][0], tq[1][1], false, q, mask);
    qto_p3(t3, t, q, mask);
    qcached_comps(tq[7][0], tq[7][1], t3, d2, q);
    qdbl(t, P4.X, P4.Y, P4.Z, q, mask);
    qto_p3(t3, t, q, mask);
    qcached_comps(tq[8][0], tq[8][1], t3, d2, q);
}

// 32-byte encoding with y (low 255 bits) < p
__device__ __forceinline__ bool enc_y_canonical(const uint32_t w[8]) {
    const uint32_t hi_ones = w[1] & w[2] & w[3] & w[4] & w[5] & w[6];
    const bool ge_p = (w[7] & 0x7fffffffu) == 0x7fffffffu && hi_ones == 0xffffffffu && w[0] >= 0xffffffedu;
    return !ge_p;
}

// Verdict of signature i, computed by the quad (every lane returns it).
// No lane leaves early: a rejected signature runs to the end with its
// verdict already cleared, so every lane of the warp meets every shuffle.
__device__ bool verify_quad(const SigBatch& a, const uint32_t* sVB, uint32_t i, uint32_t lane_q) {
    const QuadSel q = quad_sel(lane_q);
    const uint32_t mask = kQuadAll;
    uint64_t so = a.signature_offsets[i];
    uint64_t po = a.public_key_offsets[i];
    uint64_t mo = a.message_start_offsets[i];
    uint32_t m = a.message_lens[i];
    bool ok = !(so + 64 > a.packets_len || po + 32 > a.packets_len || mo + m > a.packets_len);
    if (!ok) so = po = mo = m = 0;                          // read nothing out of range

    uint32_t sig[16], pk[8];
#pragma unroll
    for (int k = 0; k < 16; k++) sig[k] = ld_u32_any(a.packets, so + 4 * k, a.packets_len);
#pragma unroll
    for (int k = 0; k < 8; k++) pk[k] = ld_u32_any(a.packets, po + 4 * k, a.packets_len);

    ok = ok && !(sig[15] & 0xf0000000u);                    // S >= 2^252
    ok = ok && !enc_is_order4(sig) && !enc_is_order4(pk);
    ok = ok && enc_y_canonical(sig);                        // R's y >= p: no canonical encoding equals it

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

    // lanes 0-1 decode A, lanes 2-3 decode R
    const CurveConsts& K = a.tables->K;
    uint32_t enc[8];
    const uint32_t take_pk = 0u - (uint32_t)(lane_q < 2);
#pragma unroll
    for (int k = 0; k < 8; k++) enc[k] = (pk[k] & take_pk) | (sig[k] & ~take_pk);
    fe dx, dy;
    const uint32_t dok = ge_decode(dx, dy, enc, K) ? 1u : 0u;
    const uint32_t okA = __shfl_sync(kQuadAll, dok, 0, 4), okR = __shfl_sync(kQuadAll, dok, 2, 4);
    ok = ok && okA && okR;
    fe ax, ay, rx, ry;
    quad_from(ax, dx, 0, mask);
    quad_from(ay, dy, 0, mask);
    quad_from(rx, dx, 2, mask);
    quad_from(ry, dy, 2, mask);
    fe_neg(ax, ax);                                          // -A

    // this lane's components of k(-A), k = 0..8
    fe tq[9][2];
    quad_table(tq, ax, ay, K.d2, q, mask);

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
        // digit i of h
        int nib = (int)(hh[7] >> 28);
        shl_words(hh, 4);
        int ci = (int)((hc >> i) & 1u);
        int cn = (i < 63) ? (int)((hc >> (i + 1)) & 1u) : 0;
        int da = nib + ci - 16 * cn;
        int ua = min(da < 0 ? -da : da, 8);
        qadd_cached(t, R, tq[ua][0], tq[ua][1], da < 0, q, mask);
        if ((i & 1) == 0) {
            qto_p3(R, t, q, mask);
            int k = i >> 1;
            int byte = (int)(ss[7] >> 24);
            shl_words(ss, 8);
            int bc = (int)((scar >> k) & 1u);
            int bn = (k < 31) ? (int)((scar >> (k + 1)) & 1u) : 0;
            int db = byte + bc - 256 * bn;
            int ub = min(db < 0 ? -db : db, VB_ENTRIES - 1);
            qadd_niels(t, R, sVB, ub, db < 0, q, lane_q, mask);
        }
        qto_p2(R.X, R.Y, R.Z, t, q, mask);
    }

    // [S]B + [h](-A) == R:  X == x_R Z (lane 0) and Y == y_R Z (lane 1)
    fe o1, prod, xz, yz;
    fe_pick4(o1, rx, ry, rx, ry, q);
    fe_mul(prod, o1, R.Z);
    quad_from(xz, prod, 0, mask);
    quad_from(yz, prod, 1, mask);
    return ok && fe_equal(R.X, xz) && fe_equal(R.Y, yz);
}
