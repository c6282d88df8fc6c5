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


def corrupt_expected(expected: np.ndarray, frac: float, seed: int):
    """Flip one bit in `frac` of the expected hashes; returns (expected', mask)."""
    rng = np.random.default_rng(seed)
    exp = expected.copy().reshape(-1, 32)
    mask = rng.random(len(exp)) < frac
    for i in np.nonzero(mask)[0]:
        bit = int(rng.integers(0, 256))
        exp[i, bit // 8] ^= np.uint8(1 << (bit % 8))
    return exp, mask
