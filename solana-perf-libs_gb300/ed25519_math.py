"""Pure-Python Ed25519 arithmetic (big integers) for building adversarial
inputs: torsion points, mixed-order points, non-canonical encodings,
undecodable encodings.  Used by the synthetic workload generator and the
tests; independent of both the CUDA library and the CPU oracle, and slow --
small numbers of points only."""
from __future__ import annotations

P = 2**255 - 19
L = 2**252 + 27742317777372353535851937790883648493
D = (-121665 * pow(121666, P - 2, P)) % P
SQRTM1 = pow(2, (P - 1) // 4, P)


def _inv(x: int) -> int:
    return pow(x, P - 2, P)


def recover_x(y: int, sign: int):
    """x with the given parity for y (mod p), None if y is not on the curve."""
    y %= P
    u = (y * y - 1) % P
    v = (D * y * y + 1) % P
    x = (u * pow(v, 3, P) * pow(u * pow(v, 7, P), (P - 5) // 8, P)) % P
    if (v * x * x - u) % P != 0:
        if (v * x * x + u) % P != 0:
            return None
        x = x * SQRTM1 % P
    if (x & 1) != sign:
        x = (-x) % P
    return x


def decode(b: bytes):
    """Decode like the reference: 255-bit y with no range check."""
    n = int.from_bytes(b, "little")
    y = n & ((1 << 255) - 1)
    x = recover_x(y, n >> 255)
    if x is None:
        return None
    return (x, y % P)


def encode(pt) -> bytes:
    x, y = pt
    return (y | ((x & 1) << 255)).to_bytes(32, "little")


def add(p1, p2):
    x1, y1 = p1
    x2, y2 = p2
    t = D * x1 * x2 * y1 * y2 % P
    x3 = (x1 * y2 + x2 * y1) * _inv(1 + t) % P
    y3 = (y1 * y2 + x1 * x2) * _inv(1 - t) % P
    return (x3, y3)


def neg(p):
    return ((-p[0]) % P, p[1])


IDENTITY = (0, 1)


def mul(k: int, pt):
    r = IDENTITY
    q = pt
    while k > 0:
        if k & 1:
            r = add(r, q)
        q = add(q, q)
        k >>= 1
    return r


BASE = (recover_x(4 * _inv(5) % P, 0), 4 * _inv(5) % P)


def order_of_torsion(pt) -> int:
    q = pt
    for k in (1, 2, 4, 8):
        if q == IDENTITY:
            return k
        q = mul(2, q) if k < 8 else q
    return 0


def torsion_generator():
    """A point of order exactly 8, derived as [L]P for curve points P."""
    y = 2
    while True:
        x = recover_x(y, 0)
        if x is not None:
            t = mul(L, (x, y))
            if mul(4, t) != IDENTITY:
                return t
        y += 1


def torsion_points():
    g = torsion_generator()
    return [mul(k, g) for k in range(8)]


def small_order_encodings():
    """Every 32-byte string that decodes to a point of order dividing 8:
    canonical encodings of the 8 torsion points with both sign bits, plus the
    non-canonical y >= p forms (y = p, p+1)."""
    out = set()
    for pt in torsion_points():
        x, y = pt
        for sign in (0, 1):
            out.add((y | (sign << 255)).to_bytes(32, "little"))
            if y + P < 2**255:
                out.add(((y + P) | (sign << 255)).to_bytes(32, "little"))
    return sorted(out)


def undecodable_encoding(rng) -> bytes:
    """A 32-byte string whose y (low 255 bits) has no matching x."""
    while True:
        b = bytes(rng.integers(0, 256, 32, dtype="uint8").tolist())
        if decode(b) is None:
            return b
