"""The half-size-scalar verification the GPU's three-warp and one-lane forms
use (csrc/half_scalar.cuh, verify_trio.cuh, verify_half.cuh), checked on the
CPU with big integers:

* the reduction, modelled step for step on its fixed word counts (9-word
  remainders and 6-word cofactors as two's complement rings, the top-64-bit
  inner loop, the exact binary step, the choice among four candidates and
  the (h, 1) fallback), gives c = d h (mod 8L) with d odd and positive for
  every h, and short pairs for random h;
* the identity behind it: for such (c, d), [S']B + [c](-A) + [d](-R) is the
  neutral point exactly when [S]B - [h]A == R, on points with small-order
  components (where a modulus of L instead of 8L would differ)."""
import hashlib
import random

import ed25519_math as E

L = E.L
M = 8 * L
R9, R6 = 2 ** 288, 2 ** 192


def _s9(x):
    x %= R9
    return x - R9 if x >> 287 else x


def _s6(x):
    x %= R6
    return x - R6 if x >> 191 else x


def half_scalars(h, max_outer=200):
    """The device algorithm (half_scalar.cuh) on Python integers."""
    r0, r1, t0, t1 = M, h, 0, 1
    outer = 0
    while r1.bit_length() > 128 and outer < max_outer:
        outer += 1
        sh = r0.bit_length() - 64
        a, b = (r0 >> sh) & (2 ** 64 - 1), (r1 >> sh) & (2 ** 64 - 1)
        lim = 32 if sh >= 97 else 129 - sh
        A, B, C, D = 1, 0, 0, 1
        n = 0
        while lim < 64 and b >> lim:
            s = a.bit_length() - b.bit_length()
            if (b << s) > a:
                s -= 1
            if s >= 32:
                break
            nA, nB = A - (C << s), B - (D << s)
            if max(abs(nA), abs(nB)) >= 2 ** 31:
                break
            a -= b << s
            A, B = nA, nB
            n += 1
            if a < b:
                a, b, A, B, C, D = b, a, C, D, A, B
        if n == 0:
            s = r0.bit_length() - r1.bit_length()
            if (r1 << s) > r0:
                s -= 1
            r0, t0 = _s9(r0 - (r1 << s)), _s6(t0 - (t1 << s))
        else:
            r0, r1 = _s9(A * r0 + B * r1), _s9(C * r0 + D * r1)
            t0, t1 = _s6(A * t0 + B * t1), _s6(C * t0 + D * t1)
            if r0 < 0:
                r0, t0 = -r0, _s6(-t0)
            if r1 < 0:
                r1, t1 = -r1, _s6(-t1)
        if r0 < r1:
            r0, r1, t0, t1 = r1, r0, t1, t0
    best = None
    for c, d in ((r1, t1), (r0, t0), (r0 + r1, t0 + t1), (r0 - r1, t0 - t1)):
        if d % 2:
            length = max(abs(c).bit_length(), abs(d).bit_length())
            if best is None or length < best[0]:
                best = (length, c, d)
    length, c, d = best
    if d < 0:
        c, d = -c, -d
    if length > 252 or d.bit_length() > 160:
        return h, 1
    return c, d


def test_reduction_congruence_and_sizes():
    rng = random.Random(11)
    hs = [0, 1, 2, 3, L - 1, L - 2, (L - 1) // 2, L // 3, 2 ** 252 - 1, 2 ** 200, 2 ** 128, 2 ** 127 + 1]
    hs += [rng.randrange(L) for _ in range(3000)]
    hs += [rng.randrange(1 << rng.randrange(1, 253)) for _ in range(500)]
    longest = 0
    for k, h in enumerate(hs):
        c, d = half_scalars(h)
        assert (c - d * h) % M == 0 and d % 2 == 1 and d > 0, h
        if 12 <= k < 3012:
            longest = max(longest, abs(c).bit_length(), d.bit_length())
    assert longest <= 150
    assert half_scalars(L - 1) == (L - 1, 1)        # no short pair with d odd: the full-length check


def test_identity_with_small_order_components():
    by = 4 * pow(5, E.P - 2, E.P) % E.P
    B = (E.recover_x(by, 0), by)
    tors = E.torsion_points()
    rng = random.Random(12)
    verdicts = set()
    for k in range(48):
        a, r = rng.randrange(1, L), rng.randrange(1, L)
        A = E.add(E.mul(a, B), tors[k % 8])
        R = E.add(E.mul(r, B), tors[(k // 8) % 8] if k % 3 == 0 else (0, 1))
        enc_a, enc_r = E.encode(A), E.encode(R)
        h = int.from_bytes(hashlib.sha512(enc_r + enc_a + bytes([k])).digest(), "little") % L
        S = (r + h * a + (1 if k % 7 == 3 else 0)) % L
        direct = E.add(E.add(E.mul(S, B), E.neg(E.mul(h, A))), E.neg(R)) == (0, 1)
        c, d = half_scalars(h)
        half = E.add(E.add(E.mul((d * S) % L, B), E.mul(c % M, E.neg(A))), E.mul(d % M, E.neg(R))) == (0, 1)
        assert direct == half, k
        verdicts.add(direct)
    assert verdicts == {True, False}
