// Edwards25519 group arithmetic (a = -1) on sm_103a, extended coordinates.
//
// Replaces the reference's ref10 group code (src/cuda-ecc-ed25519/ge.cu:
// ge_add :9, ge_p2_dbl / ge_p3_dbl, ge_madd / ge_maddsub, ge_p1p1_to_p2 /
// ge_p1p1_to_p3, ge_p3_to_cached, ge_frombytes_negate_vartime :182,
// ge_tobytes).  Same group law, own formulas and layouts:
//   ge_p3     (X:Y:Z:T)      x = X/Z, y = Y/Z, T = XY/Z
//   ge_p2     (X:Y:Z)
//   ge_done   (E, F, G, H)   a finished add/double: X = EF, Y = GH, Z = FG, T = EH
//   ge_cached (Y+X, Y-X, 2Z, 2dT)   addend with Z
//   ge_niels  (y+x, y-x, 2dxy)      affine addend (Z = 1)
#pragma once
#include "fe25519.cuh"

struct ge_p2 {
    fe X, Y, Z;
};
struct ge_p3 {
    fe X, Y, Z, T;
};
struct ge_done {
    fe E, F, G, H;
};
struct ge_cached {
    fe YpX, YmX, Z2, T2d;
};
struct ge_niels {
    fe YpX, YmX, XY2d;
};

// Curve constants, computed on the device from the curve definition at
// library start-up (see tables.cu) and passed to kernels by pointer.
struct CurveConsts {
    fe d;       // -121665/121666
    fe d2;      // 2d
    fe sqrtm1;  // 2^((p-1)/4)
};

__device__ __forceinline__ void ge_to_p2(ge_p2& r, const ge_done& c) {
    fe_mul(r.X, c.E, c.F);
    fe_mul(r.Y, c.G, c.H);
    fe_mul(r.Z, c.F, c.G);
}

__device__ __forceinline__ void ge_to_p3(ge_p3& r, const ge_done& c) {
    fe_mul(r.X, c.E, c.F);
    fe_mul(r.Y, c.G, c.H);
    fe_mul(r.Z, c.F, c.G);
    fe_mul(r.T, c.E, c.H);
}

__device__ __forceinline__ void ge_p3_identity(ge_p3& r) {
    fe_set(r.X, 0);
    fe_set(r.Y, 1);
    fe_set(r.Z, 1);
    fe_set(r.T, 0);
}

// Doubling of (X:Y:Z) (Hisil-Wong-Carter-Dawson "dbl-2008-hwcd", a = -1),
// returned with all four outputs negated, which names the same point:
//   A = X^2, B = Y^2, C = 2Z^2, E = (X+Y)^2 - A - B, G = B - A,
//   F' = C - G, H' = A + B;  X3 = E F', Y3 = G H', Z3 = F' G, T3 = E H'.
__device__ __forceinline__ void ge_dbl(ge_done& r, const fe& X, const fe& Y, const fe& Z) {
    fe a, b, c, s;
    fe_sq(a, X);
    fe_sq(b, Y);
    fe_sq(c, Z);
    fe_add(c, c, c);
    fe_add(s, X, Y);
    fe_sq(s, s);
    fe_add(r.H, a, b);
    fe_sub(r.E, s, r.H);
    fe_sub(r.G, b, a);
    fe_sub(r.F, c, r.G);
}

// p + q or p - q (neg) for a cached addend (unified addition, a = -1):
//   A = (Y1-X1)(Y2-X2), B = (Y1+X1)(Y2+X2), C = T1 2dT2, D = Z1 2Z2,
//   E = B - A, F = D - C, G = D + C, H = B + A.
// Subtracting swaps (Y2+X2, Y2-X2) and negates C, i.e. swaps F and G.
__device__ __forceinline__ void ge_add_cached(ge_done& r, const ge_p3& p, const ge_cached& q, bool neg) {
    fe ypx, ymx, qa, qb, a, b, c, d;
    fe_add(ypx, p.Y, p.X);
    fe_sub(ymx, p.Y, p.X);
    fe_select(qa, q.YmX, q.YpX, neg);
    fe_select(qb, q.YpX, q.YmX, neg);
    fe_mul(a, ymx, qa);
    fe_mul(b, ypx, qb);
    fe_mul(c, p.T, q.T2d);
    fe_mul(d, p.Z, q.Z2);
    fe_sub(r.E, b, a);
    fe_add(r.H, b, a);
    fe f, g;
    fe_sub(f, d, c);
    fe_add(g, d, c);
    fe_select(r.F, f, g, neg);
    fe_select(r.G, g, f, neg);
}

// p + q or p - q for an affine (Z = 1) addend: D = 2 Z1.
__device__ __forceinline__ void ge_add_niels(ge_done& r, const ge_p3& p, const ge_niels& q, bool neg) {
    fe ypx, ymx, qa, qb, a, b, c, d;
    fe_add(ypx, p.Y, p.X);
    fe_sub(ymx, p.Y, p.X);
    fe_select(qa, q.YmX, q.YpX, neg);
    fe_select(qb, q.YpX, q.YmX, neg);
    fe_mul(a, ymx, qa);
    fe_mul(b, ypx, qb);
    fe_mul(c, p.T, q.XY2d);
    fe_add(d, p.Z, p.Z);
    fe_sub(r.E, b, a);
    fe_add(r.H, b, a);
    fe f, g;
    fe_sub(f, d, c);
    fe_add(g, d, c);
    fe_select(r.F, f, g, neg);
    fe_select(r.G, g, f, neg);
}

__device__ __forceinline__ void ge_p3_to_cached(ge_cached& r, const ge_p3& p, const fe& d2) {
    fe_add(r.YpX, p.Y, p.X);
    fe_sub(r.YmX, p.Y, p.X);
    fe_add(r.Z2, p.Z, p.Z);
    fe_mul(r.T2d, p.T, d2);
}

__device__ __forceinline__ void ge_cached_identity(ge_cached& r) {
    fe_set(r.YpX, 1);
    fe_set(r.YmX, 1);
    fe_set(r.Z2, 2);
    fe_set(r.T2d, 0);
}

// Canonical 32-byte encoding (as 8 little-endian words) of (X:Y:Z):
// y = Y/Z reduced, bit 255 = parity of x = X/Z.
__device__ __forceinline__ void ge_encode_p2(uint32_t out[8], const fe& X, const fe& Y, const fe& Z) {
    fe zi, x, y;
    fe_invert(zi, Z);
    fe_mul(x, X, zi);
    fe_mul(y, Y, zi);
    fe cx, cy;
    fe_canon(cx, x);
    fe_canon(cy, y);
#pragma unroll
    for (int i = 0; i < 8; i++) out[i] = cy.v[i];
    out[7] |= (cx.v[0] & 1u) << 31;
}

// Decode a 32-byte encoding (8 little-endian words) to P with the
// reference's acceptance: y is the low 255 bits, never range-checked; x is
// u v^3 (u v^7)^((p-5)/8), times sqrt(-1) when v x^2 = -u; fails only when
// neither v x^2 = u nor v x^2 = -u; x is then negated so its parity equals
// bit 255 (a zero x is accepted with either bit).  Returns false on failure.
__device__ __forceinline__ bool ge_decode(fe& x, fe& y, const uint32_t w[8], const CurveConsts& K) {
    fe u, v, v3, t, one;
    fe_set(one, 1);
    fe_from_words(y, w);
    fe_sq(u, y);
    fe_mul(v, u, K.d);
    fe_sub(u, u, one);   // y^2 - 1
    fe_add(v, v, one);   // d y^2 + 1
    fe_sq(v3, v);
    fe_mul(v3, v3, v);   // v^3
    fe_sq(t, v3);
    fe_mul(t, t, v);     // v^7
    fe_mul(t, t, u);     // u v^7
    fe_pow22523(t, t);
    fe_mul(t, t, v3);
    fe_mul(x, t, u);     // candidate x
    fe vxx;
    fe_sq(vxx, x);
    fe_mul(vxx, vxx, v);
    fe chk;
    fe_sub(chk, vxx, u);
    if (!fe_iszero(chk)) {
        fe_add(chk, vxx, u);
        if (!fe_iszero(chk)) return false;
        fe_mul(x, x, K.sqrtm1);
    }
    if (fe_isodd(x) != (w[7] >> 31)) fe_neg(x, x);
    return true;
}

// y (low 255 bits of the encoding) is 0, 1, p-1, p or p+1: the points of
// order dividing 4, the only ones the reference's small-order test rejects
// (ge.cu:61-82 compares un-normalised limbs of 8P with (0,1,1,0)).
__device__ __forceinline__ bool enc_is_order4(const uint32_t w[8]) {
    uint32_t hi_ones = w[1] & w[2] & w[3] & w[4] & w[5] & w[6];
    uint32_t hi_zero = w[1] | w[2] | w[3] | w[4] | w[5] | w[6];
    uint32_t top = w[7] & 0x7fffffffu;
    bool small = (hi_zero == 0) && (top == 0) && (w[0] <= 1u);
    bool near_p = (hi_ones == 0xffffffffu) && (top == 0x7fffffffu) &&
                  (w[0] == 0xffffffecu || w[0] == 0xffffffedu || w[0] == 0xffffffeeu);
    return small || near_p;
}
