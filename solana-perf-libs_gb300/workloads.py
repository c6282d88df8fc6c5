"""Seeded synthetic workloads in the reference's data layout.

Each generator returns the packet buffer and per-signature arrays exactly as
ed25519_verify_many / ed25519_sign_many / poh_verify_many take them.  Key
generation and signing are passed in as callables (`keypairs(seeds) ->
(pk, sk)`, `sign(SigPackets) -> (n, 64)`), so the same generator feeds the
GPU library and the CPU oracle.

Workloads (sizes and distributions of the reference-facing benchmark set):
  verify_uniform   1024 packets [64-B sig][32-B pubkey][64-B message], stride
                   160, 10% of packets with one bit flipped in R, S, the
                   pubkey or the message.
  poh_uniform      4096 entries x 12500 SHA-256 steps, 5% of expected hashes
                   with one bit flipped.
  ragged_sigs      64 batches, packets per batch log-uniform in 1..8192,
                   message length uniform in 0..1232, 1..4 signatures per
                   packet at unaligned offsets; 5% each of S >= L,
                   small-order A, small-order R, undecodable A and flipped
                   message bit.
  poh_ragged       16384 entries, num_hashes log-uniform in 1..1e6, 3%
                   corrupted expected hashes.
  poh_entries      chains of Solana ledger entries: ticks (12500 hashes) and
                   transaction entries (1..64 hashes and a 32-byte mixin).
  wire_packets     Solana wire-format transactions (legacy and version-0
                   messages, 1..4 signers, random account keys, blockhash
                   and instructions) in fixed-stride packet slots with a
                   per-packet data length; a fraction corrupted (flipped
                   signature or message bit) and a fraction malformed.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

import ed25519_math as em
from cuda_crypt import SigPackets

L_INT = em.L

_SMALL_ORDER = None


def small_order_encodings() -> list:
    """The 14 encodings of points of order dividing 8 (canonical, both sign
    bits, and the non-canonical y = p, p + 1 forms)."""
    global _SMALL_ORDER
    if _SMALL_ORDER is None:
        _SMALL_ORDER = em.small_order_encodings()
    return _SMALL_ORDER


def _flip_bit(buf: np.ndarray, byte_lo: int, nbytes: int, rng) -> None:
    bit = int(rng.integers(0, nbytes * 8))
    buf[byte_lo + bit // 8] ^= np.uint8(1 << (bit % 8))


# ---------------------------------------------------------------- verify ---

def verify_uniform(keypairs, sign, n: int = 1024, msg_len: int = 64, flip_frac: float = 0.10, seed: int = 1):
    """Returns (SigPackets, corrupted_mask)."""
    rng = np.random.default_rng(seed)
    seeds = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    pk, sk = keypairs(seeds)
    msgs = rng.integers(0, 256, (n, msg_len), dtype=np.uint8)
    stride = 64 + 32 + msg_len
    idx = np.arange(n, dtype=np.uint32)
    # signing packets: [sk 64][pk 32][msg]
    spk = np.zeros((n, stride), dtype=np.uint8)
    spk[:, 0:64] = sk
    spk[:, 64:96] = pk
    spk[:, 96:] = msgs
    lens = np.full(n, msg_len, dtype=np.uint32)
    sigs = sign(SigPackets([spk.ravel()], stride, lens, idx * stride + 64, idx * stride, idx * stride + 96))
    pkt = np.zeros((n, stride), dtype=np.uint8)
    pkt[:, 0:64] = sigs
    pkt[:, 64:96] = pk
    pkt[:, 96:] = msgs
    flat = pkt.ravel()
    corrupted = rng.random(n) < flip_frac
    for i in np.nonzero(corrupted)[0]:
        region = int(rng.integers(0, 4))    # R, S, pubkey, message
        lo, nb = [(0, 32), (32, 32), (64, 32), (96, msg_len)][region]
        _flip_bit(flat, int(i) * stride + lo, nb, rng)
    sp = SigPackets([flat], stride, lens, idx * stride + 64, idx * stride, idx * stride + 96)
    return sp, corrupted


@dataclass
class RaggedSigs:
    verify: list = field(default_factory=list)       # SigPackets per batch (signatures to verify)
    sign: list = field(default_factory=list)         # SigPackets per 128-packet signing batch
    classes: list = field(default_factory=list)      # per batch: int8 class per signature


CLASS_VALID, CLASS_S_GE_L, CLASS_SMALL_A, CLASS_SMALL_R, CLASS_BAD_A, CLASS_FLIP_MSG = range(6)
RAGGED_STRIDE = 16 + 4 * 64 + 4 * 32 + 1232   # gap, signatures, pubkeys, message


def ragged_sigs(keypairs, sign, n_batches: int = 64, max_packets: int = 8192, max_msg: int = 1232,
                adversarial_frac: float = 0.05, sign_batch: int = 128, seed: int = 3,
                total_packet_cap: int | None = None) -> RaggedSigs:
    """Ragged verify batches plus the signing batches they were made from.
    `total_packet_cap` scales the workload down (tests) by capping the packet
    count of each batch."""
    rng = np.random.default_rng(seed)
    stride = RAGGED_STRIDE
    so = small_order_encodings()
    out = RaggedSigs()
    for b in range(n_batches):
        npk = int(np.floor(np.exp(rng.uniform(0.0, np.log(max_packets + 1)))))
        npk = max(1, min(max_packets, npk))
        if total_packet_cap is not None:
            npk = max(1, min(npk, total_packet_cap))
        nsig = rng.integers(1, 5, npk)
        mlen = rng.integers(0, max_msg + 1, npk)
        gap = rng.integers(0, 16, npk)
        total = int(nsig.sum())
        seeds = rng.integers(0, 256, (total, 32), dtype=np.uint8)
        pk, sk = keypairs(seeds)
        spk = np.zeros((npk, stride), dtype=np.uint8)      # signing image: sk in the sig slots (64 B each)
        vpk = np.zeros((npk, stride), dtype=np.uint8)      # verify image
        lens = np.zeros(total, dtype=np.uint32)
        pko = np.zeros(total, dtype=np.uint32)
        sgo = np.zeros(total, dtype=np.uint32)
        mso = np.zeros(total, dtype=np.uint32)
        j = 0
        for p in range(npk):
            k, m, g = int(nsig[p]), int(mlen[p]), int(gap[p])
            base = p * stride
            msg = rng.integers(0, 256, m, dtype=np.uint8)
            mo = g + 64 * 4 + 32 * 4
            for s in range(k):
                spk[p, g + 64 * s: g + 64 * s + 64] = sk[j + s]
                spk[p, g + 256 + 32 * s: g + 256 + 32 * s + 32] = pk[j + s]
                vpk[p, g + 256 + 32 * s: g + 256 + 32 * s + 32] = pk[j + s]
                lens[j + s] = m
                pko[j + s] = base + g + 256 + 32 * s
                sgo[j + s] = base + g + 64 * s
                mso[j + s] = base + mo
            spk[p, mo:mo + m] = msg
            vpk[p, mo:mo + m] = msg
            j += k
        sflat = spk.ravel()
        # sign in 128-packet batches (offsets rebased per batch)
        sigs = np.zeros((total, 64), dtype=np.uint8)
        first_sig = np.concatenate([[0], np.cumsum(nsig)]).astype(np.int64)
        for p0 in range(0, npk, sign_batch):
            p1 = min(npk, p0 + sign_batch)
            s0, s1 = int(first_sig[p0]), int(first_sig[p1])
            rebase = np.uint32(p0 * stride)
            sp = SigPackets([sflat[p0 * stride:p1 * stride].copy()], stride, lens[s0:s1].copy(),
                            pko[s0:s1] - rebase, sgo[s0:s1] - rebase, mso[s0:s1] - rebase)
            out.sign.append(sp)
            sigs[s0:s1] = sign(sp)
        vflat = vpk.ravel()
        cls = np.zeros(total, dtype=np.int8)
        for s in range(total):
            off = int(sgo[s])
            vflat[off:off + 64] = sigs[s]
        # adversarial classes
        u = rng.random(total)
        for s in range(total):
            off, po = int(sgo[s]), int(pko[s])
            c = int(u[s] // adversarial_frac) + 1 if u[s] < 4 * adversarial_frac else 0
            if c == CLASS_S_GE_L:
                S = int.from_bytes(bytes(vflat[off + 32:off + 64]), "little") + L_INT
                vflat[off + 32:off + 64] = np.frombuffer(S.to_bytes(32, "little"), dtype=np.uint8)
            elif c == CLASS_SMALL_A:
                vflat[po:po + 32] = np.frombuffer(so[int(rng.integers(0, len(so)))], dtype=np.uint8)
            elif c == CLASS_SMALL_R:
                vflat[off:off + 32] = np.frombuffer(so[int(rng.integers(0, len(so)))], dtype=np.uint8)
            elif c == 4:
                c = CLASS_BAD_A
                vflat[po:po + 32] = np.frombuffer(em.undecodable_encoding(rng), dtype=np.uint8)
            cls[s] = c
        # flipped message bit: per packet (all its signatures share the message)
        flip = rng.random(npk) < adversarial_frac
        for p in np.nonzero(flip)[0]:
            p = int(p)
            s0, s1 = int(first_sig[p]), int(first_sig[p + 1])
            m = int(lens[s0])
            if m == 0:
                continue
            _flip_bit(vflat, int(mso[s0]), m, rng)
            cls[s0:s1] = np.where(cls[s0:s1] == CLASS_VALID, CLASS_FLIP_MSG, cls[s0:s1])
        out.verify.append(SigPackets([vflat], stride, lens, pko, sgo, mso))
        out.classes.append(cls)
    return out


# -------------------------------------------------------------------- PoH ---

def poh_uniform(n: int = 4096, num_hashes: int = 12500, seed: int = 2):
    rng = np.random.default_rng(seed)
    hashes = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    counts = np.full(n, num_hashes, dtype=np.uint64)
    return hashes, counts


def poh_ragged(n: int = 16384, max_hashes: int = 1_000_000, seed: int = 4):
    rng = np.random.default_rng(seed)
    hashes = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    counts = np.floor(np.exp(rng.uniform(0.0, np.log(max_hashes + 1), n))).astype(np.uint64)
    counts = np.clip(counts, 1, max_hashes).astype(np.uint64)
    return hashes, counts


@dataclass
class PohEntries:
    """Chains of Solana ledger entries: chain c starts from start[c] and
    holds entries first[c] .. first[c + 1] - 1; entry e has num_hashes[e]
    hashes and, when has_mixin[e], the 32-byte mixin mixins[e] (the hash of
    its transactions).  `expected` (set by the caller from a recording) are
    the entry hashes."""
    start: np.ndarray
    first: np.ndarray
    num_hashes: np.ndarray
    mixins: np.ndarray
    has_mixin: np.ndarray
    expected: np.ndarray | None = None

    def entry_start(self) -> np.ndarray:
        """The hash each entry starts from: its chain's start, else the
        previous entry's expected hash."""
        out = np.zeros((len(self.num_hashes), 32), dtype=np.uint8)
        for c in range(len(self.start)):
            a, b = int(self.first[c]), int(self.first[c + 1])
            if b > a:
                out[a] = self.start[c]
                out[a + 1:b] = self.expected[a:b - 1]
        return out


def poh_entries(chains: int = 64, entries_per_chain: int = 80, tick_hashes: int = 12500, tx_frac: float = 0.8,
                max_tx_hashes: int = 64, seed: int = 12) -> PohEntries:
    """Slots of a Solana-like ledger: entries are ticks (tick_hashes hashes,
    no mixin) or transaction entries (1..max_tx_hashes hashes, a random
    mixin), `tx_frac` of them transaction entries; every chain opens with a
    mixin after zero hashes and an empty tick."""
    rng = np.random.default_rng(seed)
    n = chains * entries_per_chain
    first = np.arange(chains + 1, dtype=np.uint64) * entries_per_chain
    has_mixin = (rng.random(n) < tx_frac).astype(np.uint8)
    num_hashes = np.where(has_mixin == 1, rng.integers(1, max_tx_hashes + 1, n), tick_hashes).astype(np.uint64)
    for c in range(chains):
        e = c * entries_per_chain
        if entries_per_chain >= 3:
            num_hashes[e], has_mixin[e] = 0, 1          # a mixin with no hash before it
            num_hashes[e + 1], has_mixin[e + 1] = 0, 0  # an empty tick: the hash is unchanged
    mixins = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    start = rng.integers(0, 256, (chains, 32), dtype=np.uint8)
    return PohEntries(start, first, num_hashes, mixins, has_mixin)


def corrupt_expected(expected: np.ndarray, frac: float, seed: int):
    """Flip one bit in `frac` of the expected hashes; returns (expected', mask)."""
    rng = np.random.default_rng(seed)
    exp = expected.copy().reshape(-1, 32)
    mask = rng.random(len(exp)) < frac
    for i in np.nonzero(mask)[0]:
        bit = int(rng.integers(0, 256))
        exp[i, bit // 8] ^= np.uint8(1 << (bit % 8))
    return exp, mask


# ------------------------------------------------------- wire packets ---

PACKET_DATA_SIZE = 1232        # bytes of transaction data a packet slot holds
WIRE_STRIDE = 1280             # slot stride: data plus room for metadata

MALFORMED_KINDS = ("truncated", "count_mismatch", "zero_signatures", "few_keys", "bad_version",
                   "redundant_cu16", "len_over_stride")


def cu16(v: int) -> bytes:
    """compact-u16 encoding (7-bit groups, little-endian, top bit = more)."""
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


@dataclass
class WirePackets:
    data: np.ndarray            # (n, stride) uint8 packet slots
    stride: int
    lens: np.ndarray            # uint32 bytes of wire data per packet
    kinds: list                 # per packet: "valid", "corrupt_sig", "corrupt_msg" or a MALFORMED_KINDS entry


def _message(rng, signer_pks, versioned: bool) -> bytes:
    nsig = len(signer_pks)
    nkeys = nsig + int(rng.integers(0, 7))
    keys = [bytes(pk) for pk in signer_pks] + [rng.bytes(32) for _ in range(nkeys - nsig)]
    hdr = bytes([nsig, int(rng.integers(0, nsig)), int(rng.integers(0, nkeys - nsig + 1))])
    body = bytearray()
    if versioned:
        body.append(0x80)
    body += hdr + cu16(nkeys) + b"".join(keys) + rng.bytes(32)       # keys, recent blockhash
    nins = int(rng.integers(1, 4))
    body += cu16(nins)
    for _ in range(nins):
        nacc = int(rng.integers(0, min(nkeys, 8) + 1))
        data = rng.bytes(int(rng.integers(0, 160)))
        body += bytes([int(rng.integers(0, nkeys))]) + cu16(nacc) + \
            bytes(int(x) for x in rng.integers(0, nkeys, nacc)) + cu16(len(data)) + data
    if versioned:
        body += cu16(0)                                               # no address-table lookups
    return bytes(body)


def wire_packets(keypairs, sign, n: int = 4096, corrupt_frac: float = 0.05, malformed_frac: float = 0.03,
                 seed: int = 11, stride: int = WIRE_STRIDE, signers=(1, 1, 1, 2, 2, 3, 4)) -> WirePackets:
    """`n` packets with signer counts drawn from `signers`; signatures made
    with `keypairs` / `sign` as elsewhere."""
    rng = np.random.default_rng(seed)
    nsig = rng.choice(list(signers), n)
    total = int(nsig.sum())
    pk, sk = keypairs(rng.integers(0, 256, (total, 32), dtype=np.uint8))
    msgs, first = [], 0
    for p in range(n):
        k = int(nsig[p])
        m = _message(rng, pk[first:first + k], bool(rng.random() < 0.5))
        while len(cu16(k)) + 64 * k + len(m) > PACKET_DATA_SIZE:
            m = m[:PACKET_DATA_SIZE - len(cu16(k)) - 64 * k]
        msgs.append(m)
        first += k
    # signing image: per signature [sk 64][pk 32][message]
    simg, lens, pko, sko, mso, off = [], [], [], [], [], 0
    first = 0
    for p in range(n):
        for j in range(int(nsig[p])):
            s = first + j
            simg.append(bytes(sk[s]) + bytes(pk[s]) + msgs[p])
            sko.append(off)
            pko.append(off + 64)
            mso.append(off + 96)
            lens.append(len(msgs[p]))
            off += 96 + len(msgs[p])
        first += int(nsig[p])
    flat = np.frombuffer(b"".join(simg), dtype=np.uint8).copy()
    sigs = sign(SigPackets([flat], len(flat), np.array(lens, np.uint32), np.array(pko, np.uint32),
                           np.array(sko, np.uint32), np.array(mso, np.uint32)))
    data = np.zeros((n, stride), dtype=np.uint8)
    plen = np.zeros(n, dtype=np.uint32)
    kinds = []
    first = 0
    u = rng.random(n)
    for p in range(n):
        k = int(nsig[p])
        tx = bytearray(cu16(k) + b"".join(bytes(sigs[first + j]) for j in range(k)) + msgs[p])
        sig0 = len(cu16(k))
        msg0 = sig0 + 64 * k
        kind = "valid"
        if u[p] < malformed_frac:
            kind = MALFORMED_KINDS[int(rng.integers(0, len(MALFORMED_KINDS)))]
            if kind == "truncated":
                tx = tx[:int(rng.integers(0, msg0 + 4))]
            elif kind == "count_mismatch":
                tx[msg0 + (1 if tx[msg0] & 0x80 else 0)] = (k % 4) + 1 if k < 4 else 1
            elif kind == "zero_signatures":
                tx = bytearray(b"\x00") + tx[sig0:]
            elif kind == "few_keys":
                h = msg0 + (1 if tx[msg0] & 0x80 else 0)
                tx[h + 3] = k - 1            # fewer keys than signatures (count < 128)
            elif kind == "bad_version":
                if tx[msg0] & 0x80:
                    tx[msg0] = 0x81
                else:
                    tx = tx[:msg0] + bytearray([0x82]) + tx[msg0:]
            elif kind == "redundant_cu16":
                tx = bytearray([k | 0x80, 0x00]) + tx[sig0:]
            elif kind == "len_over_stride":
                pass
        elif u[p] < malformed_frac + corrupt_frac:
            if rng.random() < 0.5:
                kind = "corrupt_sig"
                j = int(rng.integers(0, k))
                bit = int(rng.integers(0, 512))
                tx[sig0 + 64 * j + bit // 8] ^= 1 << (bit % 8)
            else:
                kind = "corrupt_msg"
                bit = int(rng.integers(0, 8 * (len(tx) - msg0)))
                tx[msg0 + bit // 8] ^= 1 << (bit % 8)
        tx = bytes(tx[:stride])
        data[p, :len(tx)] = np.frombuffer(tx, dtype=np.uint8)
        plen[p] = len(tx) if kind != "len_over_stride" else stride + 1
        kinds.append(kind)
        first += k
    return WirePackets(data, stride, plen, kinds)


def fuzz_wire(w: WirePackets, seed: int):
    """Copies of w's packets and lengths with, per packet, one of: every
    byte random (the count byte often small), random bytes in the count and
    message-header region (version, header, key count), or an edge data
    length (0, 1, 2, 65, short by one, the stride, past the stride,
    2^32 - 1).  Returns (data, lens)."""
    rng = np.random.default_rng(seed)
    data, lens = w.data.copy(), w.lens.copy()
    n, stride = data.shape
    for i in range(n):
        r = rng.random()
        if r < 0.25:
            data[i] = rng.integers(0, 256, stride, dtype=np.uint8)
            if rng.random() < 0.6:
                data[i, 0] = rng.integers(1, 6)
            lens[i] = rng.integers(0, stride + 1)
        elif r < 0.65:
            msg0 = 1 + 64 * int(data[i, 0])
            for _ in range(int(rng.integers(1, 4))):
                pos = int(rng.integers(0, 3)) if rng.random() < 0.3 else msg0 + int(rng.integers(0, 8))
                data[i, min(pos, stride - 1)] = rng.integers(0, 256)
        elif r < 0.8:
            lens[i] = rng.choice([0, 1, 2, 65, max(0, int(lens[i]) - 1), stride, stride + 1, 0xffffffff])
    return data, lens
