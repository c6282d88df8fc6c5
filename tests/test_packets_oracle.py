"""The oracle's parse of Solana wire-format packets (oracle_parse_packets)
against an independent pure-Python parse, on crafted transactions and every
malformed kind; and the wire-packet generator's classes against the oracle's
verdicts.  CPU only."""
import numpy as np
import pytest

import workloads
from workloads import cu16


def py_cu16(b: bytes, pos: int):
    v = 0
    for i in range(3):
        if pos + i >= len(b):
            return None
        x = b[pos + i]
        v |= (x & 0x7F) << (7 * i)
        if not x & 0x80:
            if i and x == 0:
                return None
            if i == 2 and x > 3:
                return None
            return v, pos + i + 1
    return None


def py_parse(b: bytes):
    """(count, sig_off, key_off, msg_off) or count 0."""
    r = py_cu16(b, 0)
    if r is None or r[0] == 0:
        return (0,)
    n, pos = r
    so = pos
    if pos + 64 * n > len(b):
        return (0,)
    pos += 64 * n
    mo = pos
    if pos >= len(b):
        return (0,)
    if b[pos] & 0x80:
        if b[pos] & 0x7F:
            return (0,)
        pos += 1
    if pos + 3 > len(b) or b[pos] != n:
        return (0,)
    r = py_cu16(b, pos + 3)
    if r is None or r[0] < n:
        return (0,)
    k, pos = r
    if pos + 32 * k > len(b):
        return (0,)
    return (n, so, pos, mo)


def tx(nsig=1, nkeys=2, versioned=False, tail=b"\x01" * 40, count=None, req=None):
    msg = (b"\x80" if versioned else b"") + bytes([nsig if req is None else req, 0, 0]) + cu16(nkeys) + \
        bytes(range(32)) * nkeys + tail
    return cu16(nsig if count is None else count) + b"\x07" * (64 * nsig) + msg


CRAFTED = [
    tx(), tx(2, 3), tx(4, 4, True), tx(1, 1, tail=b""), tx(3, 200),        # 200 keys: 2-byte compact-u16
    tx(count=0), tx(req=2), tx(2, 1), tx(1, 2)[:100],                       # zero, mismatch, few keys, cut
    b"", b"\x01", b"\x80\x00" + tx()[1:], b"\x81\x80\x80\x01",              # empty, redundant group, 4 bytes
    tx(versioned=True).replace(b"\x80\x01\x00\x00", b"\x81\x01\x00\x00", 1),  # version 1
    tx()[:1 + 64],                                                           # no message
    tx()[:1 + 64 + 3],                                                       # header, no key count
]


def test_cu16_roundtrip():
    for v in [0, 1, 127, 128, 255, 16383, 16384, 65535]:
        e = cu16(v)
        assert py_cu16(e, 0) == (v, len(e))
    assert py_cu16(b"\xff\xff\x04", 0) is None          # above 0xffff
    assert py_cu16(b"\x80\x00", 0) is None               # redundant zero group


def test_oracle_parse_matches_python(oracle):
    stride = 8192
    data = np.zeros((len(CRAFTED), stride), dtype=np.uint8)
    lens = np.zeros(len(CRAFTED), dtype=np.uint32)
    for i, b in enumerate(CRAFTED):
        data[i, :len(b)] = np.frombuffer(b, dtype=np.uint8)
        lens[i] = len(b)
    counts, so, ko, mo, ml = oracle.parse_packets(data, stride, lens)
    for i, b in enumerate(CRAFTED):
        exp = py_parse(b)
        assert counts[i] == exp[0], i
        if exp[0]:
            base = i * stride
            assert (so[i], ko[i], mo[i], ml[i]) == (base + exp[1], base + exp[2], base + exp[3], len(b) - exp[3]), i
    assert list(counts[:5]) == [1, 2, 4, 1, 3]
    assert not counts[5:].any()


def test_len_over_stride_is_malformed(oracle):
    b = tx()
    data = np.zeros((1, 200), dtype=np.uint8)
    data[0, :len(b)] = np.frombuffer(b, dtype=np.uint8)
    assert oracle.parse_packets(data, 200, [len(b)])[0][0] == 1
    assert oracle.parse_packets(data, 200, [201])[0][0] == 0


def test_wire_generator_classes(oracle):
    w = workloads.wire_packets(oracle.create_keypairs, oracle.sign_packets, n=300, seed=21,
                               corrupt_frac=0.1, malformed_frac=0.1)
    pv, sv, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens)
    for kind, v, c, i in zip(w.kinds, pv, counts, range(len(pv))):
        b = bytes(w.data[i, :min(int(w.lens[i]), w.stride)])
        py = py_parse(b) if w.lens[i] <= w.stride else (0,)
        assert c == py[0], (i, kind)
        if kind == "valid":
            assert v == 1 and c > 0, i
        elif kind in workloads.MALFORMED_KINDS:
            assert v == 0 and c == 0, (i, kind)
        else:
            assert v == 0, (i, kind)
    assert len(set(w.kinds)) >= 6


def test_oracle_parse_matches_python_fuzzed(oracle):
    """Fuzzed packets (random bytes, corrupted headers, edge lengths): the
    oracle's C parse against the pure-Python one, packet by packet."""
    w = workloads.wire_packets(oracle.create_keypairs, oracle.sign_packets, n=800, seed=301, corrupt_frac=0.0,
                               malformed_frac=0.0)
    data, lens = workloads.fuzz_wire(w, 301)
    counts, so, ko, mo, ml = oracle.parse_packets(data, w.stride, lens)
    parsed = 0
    for i in range(len(lens)):
        n = int(lens[i])
        exp = (0,) if n > w.stride else py_parse(bytes(data[i, :n]))
        assert counts[i] == exp[0], i
        if exp[0]:
            parsed += 1
            base = i * w.stride
            assert (so[i], ko[i], mo[i], ml[i]) == (base + exp[1], base + exp[2], base + exp[3], n - exp[3]), i
    assert 200 < parsed < 700
