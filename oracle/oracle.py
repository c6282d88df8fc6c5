"""ctypes access to the CPU oracle (oracle/liboracle.so) and, where it was
built, to the reference compiled from source (oracle/_ref/libref_crypt.so).

Test infrastructure only: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by ``bench.py`` for the timed CPU baseline.  The product
library never loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_crypt.so")

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def build_oracle() -> None:
    """Compile oracle/crypt_oracle.c (gcc; seconds)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def build_ref(ref_root: str | None = None) -> bool:
    """Compile the reference's host code from its own sources when the tree is
    present (x86_64 only).  The tree is `ref_root`, else $REF_ROOT, else
    /root/reference.  Returns True when oracle/_ref is usable."""
    ref_root = ref_root or os.environ.get("REF_ROOT", "/root/reference")
    if os.path.exists(REF_SO):
        return True
    if not os.path.isdir(ref_root):
        return False
    repo = os.path.dirname(HERE)
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "ref.mk"), f"REF={ref_root}", "-j2"],
                   cwd=repo, check=True)
    return os.path.exists(REF_SO)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _bytes_arg(b) -> ctypes.Array:
    b = bytes(b)
    return (ctypes.c_uint8 * max(1, len(b))).from_buffer_copy(b if b else b"\0")


class _Lib:
    def __init__(self, path: str):
        self.lib = ctypes.CDLL(path)


class Oracle(_Lib):
    """The C restatement (crypt_oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        super().__init__(path)
        L = self.lib
        L.oracle_init.restype = None
        L.oracle_init()
        L.oracle_ed25519_verify.restype = ctypes.c_int
        L.oracle_ed25519_verify.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p]
        L.oracle_ed25519_sign.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p, _u8p]
        L.oracle_ed25519_create_keypair.argtypes = [_u8p, _u8p, _u8p]
        L.oracle_get_checked_scalar.argtypes = [_u8p, _u8p]
        L.oracle_check_packed_ge_small_order.argtypes = [_u8p]
        L.oracle_sc_reduce.argtypes = [_u8p, _u8p]
        L.oracle_sc_muladd.argtypes = [_u8p, _u8p, _u8p, _u8p]
        L.oracle_scalarmult_base.argtypes = [_u8p, _u8p]
        L.oracle_double_scalarmult.argtypes = [_u8p, _u8p, _u8p, _u8p]
        L.oracle_point_roundtrip.argtypes = [_u8p, _u8p]
        L.oracle_point_add.argtypes = [_u8p, _u8p, _u8p]
        L.oracle_sha512.argtypes = [_u8p, ctypes.c_size_t, _u8p]
        L.oracle_sha256.argtypes = [_u8p, ctypes.c_size_t, _u8p]
        L.oracle_poh_chain.argtypes = [_u8p, ctypes.c_uint64]
        L.oracle_verify_many.argtypes = [_u8p, ctypes.c_uint32, _u32p, _u32p, _u32p, _u32p, _u8p, ctypes.c_int]
        L.oracle_sign_many.argtypes = [_u8p, ctypes.c_uint32, _u32p, _u32p, _u32p, _u32p, _u8p, ctypes.c_int]
        L.oracle_poh_verify_many.argtypes = [_u8p, _u64p, ctypes.c_size_t, ctypes.c_int]
        L.oracle_create_keypairs.argtypes = [_u8p, _u8p, _u8p, ctypes.c_size_t, ctypes.c_int]
        L.oracle_parse_packets.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_uint32, _u32p] + [_u32p] * 5
        L.oracle_parse_packets.restype = None
        L.oracle_poh_entry.argtypes = [_u8p, ctypes.c_uint64, _u8p]
        L.oracle_poh_verify_entries.argtypes = [_u8p, _u64p, _u8p, _u8p, _u8p, ctypes.c_size_t, _u8p, _u8p,
                                                ctypes.c_int]
        L.oracle_poh_record.argtypes = [_u8p, ctypes.c_size_t, _u64p, _u64p, _u8p, _u8p, _u8p]

    # ---- single items -----------------------------------------------------
    def create_keypair(self, seed: bytes):
        pk = (ctypes.c_uint8 * 32)()
        sk = (ctypes.c_uint8 * 64)()
        self.lib.oracle_ed25519_create_keypair(pk, sk, _bytes_arg(seed))
        return bytes(pk), bytes(sk)

    def sign(self, msg: bytes, pk: bytes, sk: bytes) -> bytes:
        sig = (ctypes.c_uint8 * 64)()
        self.lib.oracle_ed25519_sign(sig, _bytes_arg(msg), len(msg), _bytes_arg(pk), _bytes_arg(sk))
        return bytes(sig)

    def verify(self, sig: bytes, msg: bytes, pk: bytes) -> int:
        return self.lib.oracle_ed25519_verify(_bytes_arg(sig), _bytes_arg(msg), len(msg), _bytes_arg(pk))

    def get_checked_scalar(self, s: bytes) -> int:
        out = (ctypes.c_uint8 * 32)()
        return self.lib.oracle_get_checked_scalar(out, _bytes_arg(s))

    def check_packed_ge_small_order(self, p: bytes) -> int:
        return self.lib.oracle_check_packed_ge_small_order(_bytes_arg(p))

    def sc_reduce(self, h64: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.oracle_sc_reduce(out, _bytes_arg(h64))
        return bytes(out)

    def sc_muladd(self, a: bytes, b: bytes, c: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.oracle_sc_muladd(out, _bytes_arg(a), _bytes_arg(b), _bytes_arg(c))
        return bytes(out)

    def scalarmult_base(self, a: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.oracle_scalarmult_base(out, _bytes_arg(a))
        return bytes(out)

    def double_scalarmult(self, a: bytes, A: bytes, b: bytes):
        out = (ctypes.c_uint8 * 32)()
        ok = self.lib.oracle_double_scalarmult(out, _bytes_arg(a), _bytes_arg(A), _bytes_arg(b))
        return bytes(out) if ok else None

    def point_roundtrip(self, p: bytes):
        out = (ctypes.c_uint8 * 32)()
        ok = self.lib.oracle_point_roundtrip(out, _bytes_arg(p))
        return bytes(out) if ok else None

    def point_add(self, a: bytes, b: bytes):
        out = (ctypes.c_uint8 * 32)()
        ok = self.lib.oracle_point_add(out, _bytes_arg(a), _bytes_arg(b))
        return bytes(out) if ok else None

    def sha512(self, m: bytes) -> bytes:
        out = (ctypes.c_uint8 * 64)()
        self.lib.oracle_sha512(_bytes_arg(m), len(m), out)
        return bytes(out)

    def sha256(self, m: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.oracle_sha256(_bytes_arg(m), len(m), out)
        return bytes(out)

    def poh_chain(self, h: bytes, n: int) -> bytes:
        buf = _bytes_arg(h)
        self.lib.oracle_poh_chain(buf, n)
        return bytes(buf)

    # ---- batch forms (same argument meaning as the C ABI) ------------------
    def create_keypairs(self, seeds: np.ndarray, nthreads: int = 0):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint8).reshape(-1, 32)
        n = len(seeds)
        pk = np.zeros((n, 32), dtype=np.uint8)
        sk = np.zeros((n, 64), dtype=np.uint8)
        self.lib.oracle_create_keypairs(_ptr(seeds, _u8p), _ptr(pk, _u8p), _ptr(sk, _u8p), n,
                                        nthreads or os.cpu_count() or 1)
        return pk, sk

    def sign_packets(self, sp, nthreads: int = 0) -> np.ndarray:
        """sign_many over a SigPackets (the library's batch description)."""
        return self.sign_many(sp.concatenated(), sp.message_lens, sp.public_key_offsets, sp.signature_offsets,
                              sp.message_start_offsets, nthreads or os.cpu_count() or 1)

    def verify_packets(self, sp, nthreads: int = 0) -> np.ndarray:
        return self.verify_many(sp.concatenated(), sp.message_lens, sp.public_key_offsets, sp.signature_offsets,
                                sp.message_start_offsets, nthreads or os.cpu_count() or 1)

    def verify_many(self, packets: np.ndarray, message_lens, public_key_offsets, signature_offsets,
                    message_start_offsets, nthreads: int = 1) -> np.ndarray:
        n = len(message_lens)
        out = np.zeros(n, dtype=np.uint8)
        arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
                (message_lens, public_key_offsets, signature_offsets, message_start_offsets)]
        packets = np.ascontiguousarray(packets, dtype=np.uint8)
        self.lib.oracle_verify_many(_ptr(packets, _u8p), n, *[_ptr(a, _u32p) for a in arrs],
                                    _ptr(out, _u8p), nthreads)
        return out

    def sign_many(self, packets: np.ndarray, message_lens, public_key_offsets, private_key_offsets,
                  message_start_offsets, nthreads: int = 1) -> np.ndarray:
        n = len(message_lens)
        out = np.zeros((n, 64), dtype=np.uint8)
        arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
                (message_lens, public_key_offsets, private_key_offsets, message_start_offsets)]
        packets = np.ascontiguousarray(packets, dtype=np.uint8)
        self.lib.oracle_sign_many(_ptr(packets, _u8p), n, *[_ptr(a, _u32p) for a in arrs],
                                  _ptr(out, _u8p), nthreads)
        return out

    def parse_packets(self, data: np.ndarray, stride: int, lens):
        """Per packet: (counts, signature, key and message offsets, message
        lengths), offsets absolute in `data` (oracle_parse_packets)."""
        lens = np.ascontiguousarray(lens, dtype=np.uint32)
        n = len(lens)
        data = np.ascontiguousarray(data, dtype=np.uint8).ravel()
        outs = [np.zeros(n, dtype=np.uint32) for _ in range(5)]
        self.lib.oracle_parse_packets(_ptr(data, _u8p), ctypes.c_uint64(stride), n, _ptr(lens, _u32p),
                                      *[_ptr(a, _u32p) for a in outs])
        return tuple(outs)

    def wire_offsets(self, data: np.ndarray, stride: int, lens):
        """The reference's four per-signature arrays for a packet batch, plus
        the per-packet counts: (counts, message_lens, public_key_offsets,
        signature_offsets, message_start_offsets)."""
        counts, so, ko, mo, ml = self.parse_packets(data, stride, lens)
        total = int(counts.sum())
        pkt = np.repeat(np.arange(len(counts)), counts)
        first = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
        idx = np.arange(total) - first[pkt]
        return (counts, ml[pkt].astype(np.uint32), (ko[pkt] + 32 * idx).astype(np.uint32),
                (so[pkt] + 64 * idx).astype(np.uint32), mo[pkt].astype(np.uint32))

    def verify_wire_packets(self, data: np.ndarray, stride: int, lens, nthreads: int = 0):
        """(per-packet verdicts, per-signature verdicts, counts): a packet
        passes when it parses and every one of its signatures verifies."""
        counts, ml, ko, so, mo = self.wire_offsets(data, stride, lens)
        sig = self.verify_many(np.ascontiguousarray(data, dtype=np.uint8).ravel(), ml, ko, so, mo,
                               nthreads or os.cpu_count() or 1)
        pkt = np.repeat(np.arange(len(counts)), counts)
        bad = np.zeros(len(counts), dtype=np.int64)
        np.add.at(bad, pkt, (sig == 0).astype(np.int64))
        return ((counts > 0) & (bad == 0)).astype(np.uint8), sig, counts

    # ---- PoH entries with transaction mixins (Solana ledger entries) ---------
    def poh_entry(self, h: bytes, num_hashes: int, mixin: bytes | None) -> bytes:
        buf = _bytes_arg(h)
        self.lib.oracle_poh_entry(buf, num_hashes, _bytes_arg(mixin) if mixin is not None else None)
        return bytes(buf)

    def poh_verify_entries(self, start, num_hashes, mixins, has_mixin, expected, nthreads: int = 0):
        """(ok per entry, computed entry hashes)."""
        start = np.ascontiguousarray(start, dtype=np.uint8).reshape(-1, 32)
        n = len(start)
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        mx = np.ascontiguousarray(mixins, dtype=np.uint8).reshape(-1, 32)
        hm = np.ascontiguousarray(has_mixin, dtype=np.uint8)
        ex = np.ascontiguousarray(expected, dtype=np.uint8).reshape(-1, 32)
        ok = np.zeros(n, dtype=np.uint8)
        out = np.zeros((n, 32), dtype=np.uint8)
        self.lib.oracle_poh_verify_entries(_ptr(start, _u8p), _ptr(nh, _u64p), _ptr(mx, _u8p), _ptr(hm, _u8p),
                                           _ptr(ex, _u8p), n, _ptr(ok, _u8p), _ptr(out, _u8p),
                                           nthreads or os.cpu_count() or 1)
        return ok, out

    def poh_record(self, start, first, num_hashes, mixins, has_mixin):
        """(entry hashes, final hash per chain); chain c runs entries
        first[c] .. first[c + 1] - 1."""
        h = np.array(start, dtype=np.uint8, copy=True).reshape(-1, 32)
        fi = np.ascontiguousarray(first, dtype=np.uint64)
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        mx = np.ascontiguousarray(mixins, dtype=np.uint8).reshape(-1, 32)
        hm = np.ascontiguousarray(has_mixin, dtype=np.uint8)
        out = np.zeros((len(nh), 32), dtype=np.uint8)
        self.lib.oracle_poh_record(_ptr(h, _u8p), len(h), _ptr(fi, _u64p), _ptr(nh, _u64p), _ptr(mx, _u8p),
                                   _ptr(hm, _u8p), _ptr(out, _u8p))
        return out, h

    def poh_verify_many(self, hashes: np.ndarray, num_hashes, nthreads: int = 1) -> np.ndarray:
        """Returns the final hashes (the input array is not modified)."""
        h = np.array(hashes, dtype=np.uint8, copy=True).reshape(-1, 32)
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        self.lib.oracle_poh_verify_many(_ptr(h, _u8p), _ptr(nh, _u64p), len(nh), nthreads)
        return h


class RefLib(_Lib):
    """The reference's own host functions compiled from its sources."""

    def __init__(self, path: str = REF_SO):
        super().__init__(path)
        L = self.lib
        L.ed25519_verify.restype = ctypes.c_int
        L.ed25519_verify.argtypes = [_u8p, _u8p, ctypes.c_uint32, _u8p]
        L.ed25519_sign.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p, _u8p]
        L.ed25519_create_keypair.argtypes = [_u8p, _u8p, _u8p]
        L.ed25519_get_checked_scalar.argtypes = [_u8p, _u8p]
        L.ed25519_check_packed_ge_small_order.argtypes = [_u8p]
        L.ref_sc_reduce.argtypes = [_u8p]
        L.ref_sc_muladd.argtypes = [_u8p, _u8p, _u8p, _u8p]
        L.ref_scalarmult_base.argtypes = [_u8p, _u8p]
        L.ref_double_scalarmult.argtypes = [_u8p, _u8p, _u8p, _u8p]
        L.ref_poh_chain.argtypes = [_u8p, ctypes.c_ulonglong]

    def create_keypair(self, seed: bytes):
        pk = (ctypes.c_uint8 * 32)()
        sk = (ctypes.c_uint8 * 64)()
        self.lib.ed25519_create_keypair(pk, sk, _bytes_arg(seed))
        return bytes(pk), bytes(sk)

    def sign(self, msg: bytes, pk: bytes, sk: bytes) -> bytes:
        sig = (ctypes.c_uint8 * 64)()
        self.lib.ed25519_sign(sig, _bytes_arg(msg), len(msg), _bytes_arg(pk), _bytes_arg(sk))
        return bytes(sig)

    def verify(self, sig: bytes, msg: bytes, pk: bytes) -> int:
        return self.lib.ed25519_verify(_bytes_arg(sig), _bytes_arg(msg), len(msg), _bytes_arg(pk))

    def get_checked_scalar(self, s: bytes) -> int:
        out = (ctypes.c_uint8 * 32)()
        return self.lib.ed25519_get_checked_scalar(out, _bytes_arg(s))

    def check_packed_ge_small_order(self, p: bytes) -> int:
        return self.lib.ed25519_check_packed_ge_small_order(_bytes_arg(p))

    def sc_reduce(self, h64: bytes) -> bytes:
        buf = _bytes_arg(h64)
        self.lib.ref_sc_reduce(buf)
        return bytes(buf)[:32]

    def sc_muladd(self, a: bytes, b: bytes, c: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.ref_sc_muladd(out, _bytes_arg(a), _bytes_arg(b), _bytes_arg(c))
        return bytes(out)

    def scalarmult_base(self, a: bytes) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        self.lib.ref_scalarmult_base(out, _bytes_arg(a))
        return bytes(out)

    def double_scalarmult(self, a: bytes, A: bytes, b: bytes):
        out = (ctypes.c_uint8 * 32)()
        ok = self.lib.ref_double_scalarmult(out, _bytes_arg(a), _bytes_arg(A), _bytes_arg(b))
        return bytes(out) if ok else None

    def poh_chain(self, h: bytes, n: int) -> bytes:
        buf = _bytes_arg(h)
        self.lib.ref_poh_chain(buf, n)
        return bytes(buf)


_oracle = None


def get_oracle() -> Oracle:
    global _oracle
    if _oracle is None:
        _oracle = Oracle()
    return _oracle


def get_ref():
    """The compiled reference, or None where it is not available."""
    if os.path.exists(REF_SO):
        return RefLib()
    return None
