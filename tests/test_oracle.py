"""The CPU oracle pinned against the reference: its golden vectors, the
reference's own host code (where it compiles, i.e. here on x86_64), and
hashlib for the hash functions."""
import hashlib
import os

import numpy as np
import pytest

import ed25519_math as em


def test_poh_golden_332(oracle, golden_poh):
    hashes = np.array([list(bytes.fromhex(h)) for h in golden_poh["hashes"]], dtype=np.uint8)
    out = oracle.poh_verify_many(hashes, golden_poh["num_hashes"], nthreads=os.cpu_count() or 1)
    exp = [bytes.fromhex(h) for h in golden_poh["expected"]]
    assert [bytes(r) for r in out] == exp
    assert len(exp) == 129 and sorted(set(golden_poh["num_hashes"])) == [2451, 16901, 19353]


def test_hashes_vs_hashlib(oracle):
    rng = np.random.default_rng(5)
    for n in [0, 1, 55, 56, 63, 64, 111, 112, 119, 120, 127, 128, 129, 300, 1232]:
        m = bytes(rng.integers(0, 256, n, dtype=np.uint8).tolist())
        assert oracle.sha512(m) == hashlib.sha512(m).digest()
        assert oracle.sha256(m) == hashlib.sha256(m).digest()
    h = bytes(32)
    x = h
    for _ in range(100):
        x = hashlib.sha256(x).digest()
    assert oracle.poh_chain(h, 100) == x
    assert oracle.poh_chain(h, 0) == h


def test_ed25519_golden(oracle, golden_ed):
    for k in golden_ed["keys"]:
        pk, sk = oracle.create_keypair(bytes.fromhex(k["seed"]))
        assert pk.hex() == k["pk"] and sk.hex() == k["sk"]
    bad = []
    for c in golden_ed["verify"]:
        got = oracle.verify(bytes.fromhex(c["sig"]), bytes.fromhex(c["msg"]), bytes.fromhex(c["pk"]))
        if got != c["valid"]:
            bad.append(c["kind"])
    assert not bad
    for c in golden_ed["small_order"]:
        assert oracle.check_packed_ge_small_order(bytes.fromhex(c["point"])) == c["result"], c
    for c in golden_ed["checked_scalar"]:
        assert oracle.get_checked_scalar(bytes.fromhex(c["scalar"])) == c["result"], c
    # signatures in the golden set were made by the reference: re-sign valid ones
    keys = {k["pk"]: k for k in golden_ed["keys"]}
    for c in golden_ed["verify"]:
        if c["kind"] == "valid":
            k = keys[c["pk"]]
            assert oracle.sign(bytes.fromhex(c["msg"]), bytes.fromhex(k["pk"]), bytes.fromhex(k["sk"])).hex() == c["sig"]


def test_small_order_set():
    enc = em.small_order_encodings()
    assert len(enc) == 14
    orders = sorted(em.order_of_torsion(em.decode(e)) for e in enc)
    assert orders.count(8) == 4 and orders.count(4) == 4


# ---- against the reference's own code (skipped where it does not build) ----

def test_vs_ref_scalars(oracle, ref):
    rng = np.random.default_rng(6)
    for _ in range(3000):
        x = bytes(rng.integers(0, 256, 64, dtype=np.uint8).tolist())
        assert oracle.sc_reduce(x) == ref.sc_reduce(x)
        a, b, c = (bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist()) for _ in range(3))
        assert oracle.sc_muladd(a, b, c) == ref.sc_muladd(a, b, c)
    for v in [0, 1, em.L - 1, em.L, em.L + 1, 2**512 - 1, em.L * em.L, 2**256 - 1]:
        xb = (v % 2**512).to_bytes(64, "little")
        assert oracle.sc_reduce(xb) == ref.sc_reduce(xb)


def test_vs_ref_sign_verify(oracle, ref):
    rng = np.random.default_rng(7)
    for i in range(400):
        seed = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
        pk, sk = oracle.create_keypair(seed)
        assert (pk, sk) == ref.create_keypair(seed)
        m = bytes(rng.integers(0, 256, int(rng.integers(0, 400)), dtype=np.uint8).tolist())
        s1 = oracle.sign(m, pk, sk)
        assert s1 == ref.sign(m, pk, sk)
        skr = bytes(rng.integers(0, 256, 64, dtype=np.uint8).tolist())     # unclamped key bytes
        assert oracle.sign(m, pk, skr) == ref.sign(m, pk, skr)
        for _ in range(3):
            s2 = bytearray(s1)
            bit = int(rng.integers(0, 512))
            s2[bit // 8] ^= 1 << (bit % 8)
            assert oracle.verify(bytes(s2), m, pk) == ref.verify(bytes(s2), m, pk)


def test_vs_ref_long_messages(oracle, ref):
    """Messages far past a packet (many SHA-512 blocks): sign, verify, and
    verify with a late or middle byte altered, against the reference."""
    rng = np.random.default_rng(71)
    for n in (1232, 1233, 2047, 4103, 65647, 200003):
        seed = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
        pk, sk = oracle.create_keypair(seed)
        m = rng.bytes(n)
        s = oracle.sign(m, pk, sk)
        assert s == ref.sign(m, pk, sk), n
        assert oracle.verify(s, m, pk) == ref.verify(s, m, pk) == 1, n
        for pos in (n - 1, n // 2):
            bad = bytearray(m)
            bad[pos] ^= 0x40
            assert oracle.verify(s, bytes(bad), pk) == ref.verify(s, bytes(bad), pk) == 0, (n, pos)


def test_vs_ref_decoding(oracle, ref):
    rng = np.random.default_rng(8)
    for _ in range(20000):
        e = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
        assert oracle.check_packed_ge_small_order(e) == ref.check_packed_ge_small_order(e)
    for e in em.small_order_encodings():
        assert oracle.check_packed_ge_small_order(e) == ref.check_packed_ge_small_order(e)
    for j in range(19):
        for s in (0, 1):
            e = ((em.P + j) | (s << 255)).to_bytes(32, "little")
            assert oracle.check_packed_ge_small_order(e) == ref.check_packed_ge_small_order(e)


def test_vs_ref_double_scalarmult(oracle, ref):
    rng = np.random.default_rng(9)
    tors = em.torsion_points()
    for i in range(200):
        pk, _ = oracle.create_keypair(bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist()))
        A = em.encode(em.add(em.decode(pk), tors[i % 8]))
        # the verify domain: a = h mod L, b = S < 2^252 (the reference's
        # sliding-window recoding drops carries out of bit 255 for larger a)
        a = (int.from_bytes(bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist()), "little") % em.L).to_bytes(32, "little")
        b = bytearray(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
        b[31] &= 0x0F
        assert oracle.double_scalarmult(a, A, bytes(b)) == ref.double_scalarmult(a, A, bytes(b))


def test_vs_ref_poh(oracle, ref):
    rng = np.random.default_rng(10)
    for n in [0, 1, 2, 17, 1000]:
        h = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
        assert oracle.poh_chain(h, n) == ref.poh_chain(h, n)


def _digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_oracle_matches_reference_config_digests(oracle):
    """The full-size workload digests (made by the reference's host code)
    reproduced by the oracle: the 1,024-packet verify, 4096 x 12,500 PoH and
    the 64-batch ragged verify + 359 signing jobs.  The 16,384-chain ragged
    PoH (1.17 G hashes) is checked on the GPU only."""
    import json
    import workloads
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "config_digests.json")) as f:
        g = json.load(f)
    n = os.cpu_count() or 1
    sp, _ = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=1024, seed=1)
    assert _digest(sp.concatenated()) == g["verify_1024"]["input_sha256"]
    assert _digest(oracle.verify_packets(sp, n)) == g["verify_1024"]["verdicts_sha256"]
    h, c = workloads.poh_uniform(4096, 12500, seed=2)
    assert _digest(oracle.poh_verify_many(h, c, n)) == g["poh_uniform"]["final_sha256"]
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, seed=3)
    gr = g["ragged_sigs"]
    assert _digest(*[s.concatenated() for s in rs.verify]) == gr["verify_input_sha256"]
    assert _digest(np.concatenate([oracle.verify_packets(s, n) for s in rs.verify])) == gr["verdicts_sha256"]
    assert _digest(*[oracle.sign_packets(s, n) for s in rs.sign]) == gr["signatures_sha256"]
    h, c = workloads.poh_ragged(16384, 1_000_000, seed=4)
    assert _digest(h, c) == g["poh_ragged"]["input_sha256"]


def test_poh_entries_oracle_vs_hashlib(oracle):
    """The ledger-entry rule (tick: num_hashes plain hashes; mixin:
    max(num_hashes, 1) - 1 plain hashes then SHA-256(h || mixin)) restated
    in the oracle, against hashlib; recording and verification forms agree
    with it."""
    import workloads
    rng = np.random.default_rng(31)

    def entry(h, n, m):
        if m is None:
            for _ in range(n):
                h = hashlib.sha256(h).digest()
            return h
        for _ in range(max(n, 1) - 1):
            h = hashlib.sha256(h).digest()
        return hashlib.sha256(h + m).digest()

    h = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
    m = bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())
    for n in (0, 1, 2, 3, 64, 300):
        assert oracle.poh_entry(h, n, None) == entry(h, n, None)
        assert oracle.poh_entry(h, n, m) == entry(h, n, m)
    w = workloads.poh_entries(chains=5, entries_per_chain=12, tick_hashes=40, seed=32)
    rec, last = oracle.poh_record(w.start, w.first, w.num_hashes, w.mixins, w.has_mixin)
    for c in range(5):
        x = bytes(w.start[c])
        for e in range(int(w.first[c]), int(w.first[c + 1])):
            x = entry(x, int(w.num_hashes[e]), bytes(w.mixins[e]) if w.has_mixin[e] else None)
            assert bytes(rec[e]) == x
        assert bytes(last[c]) == x
    w.expected = rec
    exp = rec.copy()
    exp[[3, 17, 40]] ^= 1
    ok, out = oracle.poh_verify_entries(w.entry_start(), w.num_hashes, w.mixins, w.has_mixin, exp, 4)
    assert np.array_equal(out, rec)
    assert [i for i in range(len(ok)) if not ok[i]] == [3, 17, 40]
