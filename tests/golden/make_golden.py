#!/usr/bin/env python3
"""Regenerates the golden fixtures in this directory from the reference.

  poh_332.json       the reference's own PoH test vectors
                     (src/poh-verify-test/test_hashes_332_129,
                     test_num_hashes_arr_332, test_hashes_output_332),
                     re-encoded as hex.
  ed25519_ref.json   Ed25519 keypair/sign/verify vectors whose expected
                     outputs were computed by the reference's own host code
                     (oracle/_ref, compiled from the reference sources by
                     oracle/ref.mk): random messages of 0..300 bytes, every
                     small-order encoding, mixed-order keys, S >= L, S with
                     the top bits set, undecodable keys, bit flips, and
                     order-8 forgeries that the reference accepts.

Needs the reference tree (default /root/reference) and an x86_64 host.
Run from the repository root:  python3 tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "solana-perf-libs_gb300"))

from oracle.oracle import RefLib, build_ref  # noqa: E402
import ed25519_math as em  # noqa: E402

REF = os.environ.get("REF_ROOT", "/root/reference")
OUT = os.path.dirname(os.path.abspath(__file__))


def poh_fixture():
    d = os.path.join(REF, "src", "poh-verify-test")
    inp = [int(x) for x in open(os.path.join(d, "test_hashes_332_129")).read().split()]
    cnt = [int(x) for x in open(os.path.join(d, "test_num_hashes_arr_332")).read().split()]
    n_bytes = int(open(os.path.join(d, "test_num_elems_332")).read().split()[0])
    exp = [int(x) for x in open(os.path.join(d, "test_hashes_output_332")).read().split()]
    assert n_bytes == len(inp) == len(exp) and n_bytes % 32 == 0
    n = n_bytes // 32
    cnt = cnt[:n]
    return {
        "source": "src/poh-verify-test/{test_hashes_332_129,test_num_hashes_arr_332,test_hashes_output_332}",
        "hashes": [bytes(inp[32 * i:32 * i + 32]).hex() for i in range(n)],
        "num_hashes": cnt,
        "expected": [bytes(exp[32 * i:32 * i + 32]).hex() for i in range(n)],
    }


def ed25519_fixture(ref: RefLib):
    rng = np.random.default_rng(20260101)

    def rb(k):
        return bytes(rng.integers(0, 256, k, dtype=np.uint8).tolist())

    keys, cases = [], []
    for i in range(48):
        seed = rb(32)
        pk, sk = ref.create_keypair(seed)
        keys.append({"seed": seed.hex(), "pk": pk.hex(), "sk": sk.hex()})
    small = em.small_order_encodings()
    tors = em.torsion_points()

    def add(kind, sig, msg, pk):
        cases.append({"kind": kind, "sig": sig.hex(), "msg": msg.hex(), "pk": pk.hex(),
                      "valid": int(ref.verify(sig, msg, pk))})

    lens = [0, 1, 31, 32, 33, 47, 48, 63, 64, 65, 111, 112, 127, 128, 129, 175, 176, 239, 240, 300]
    for i, k in enumerate(keys):
        pk, sk = bytes.fromhex(k["pk"]), bytes.fromhex(k["sk"])
        msg = rb(lens[i % len(lens)])
        sig = ref.sign(msg, pk, sk)
        add("valid", sig, msg, pk)
        S = int.from_bytes(sig[32:], "little")
        add("s_plus_l", sig[:32] + (S + em.L).to_bytes(32, "little"), msg, pk)
        add("s_top_bits", sig[:32] + (S | (int(rng.integers(1, 16)) << 252)).to_bytes(32, "little"), msg, pk)
        add("small_a", sig, msg, small[i % len(small)])
        add("small_r", small[(i + 3) % len(small)] + sig[32:], msg, pk)
        add("mixed_a", sig, msg, em.encode(em.add(em.decode(pk), tors[1 + i % 7])))
        add("mixed_r", em.encode(em.add(em.decode(sig[:32]), tors[1 + (i + 2) % 7])) + sig[32:], msg, pk)
        add("bad_a", sig, msg, em.undecodable_encoding(rng))
        for _ in range(2):
            s2 = bytearray(sig)
            bit = int(rng.integers(0, 512))
            s2[bit // 8] ^= 1 << (bit % 8)
            add("flip_sig", bytes(s2), msg, pk)
        if msg:
            m2 = bytearray(msg)
            bit = int(rng.integers(0, 8 * len(msg)))
            m2[bit // 8] ^= 1 << (bit % 8)
            add("flip_msg", sig, bytes(m2), pk)
    # S = 0 forgeries with an order-8 key: accepted when R = [-h]A
    order8 = [t for t in tors if em.order_of_torsion(t) == 8]
    forged = 0
    while forged < 8:
        A = order8[int(rng.integers(0, len(order8)))]
        R = tors[int(rng.integers(0, 8))]
        msg = rb(16)
        sig = em.encode(R) + bytes(32)
        ok = ref.verify(sig, msg, em.encode(A))
        if ok:
            forged += 1
            add("order8_forgery", sig, msg, em.encode(A))
    # single-call helpers
    points = small + [bytes.fromhex(k["pk"]) for k in keys[:8]] + [em.undecodable_encoding(rng) for _ in range(4)]
    points += [((em.P + j) | (s << 255)).to_bytes(32, "little") for j in range(19) for s in (0, 1)]
    small_order = [{"point": p.hex(), "result": int(ref.check_packed_ge_small_order(p))} for p in points]
    scalars = [(em.L - 1), em.L, 2**252, 2**252 - 1, 2**255, 2**256 - 1, 0, 1]
    checked = [{"scalar": s.to_bytes(32, "little").hex(), "result": int(ref.get_checked_scalar(s.to_bytes(32, "little")))}
               for s in scalars]
    return {"source": "expected outputs from the reference host code (oracle/_ref)",
            "keys": keys, "verify": cases, "small_order": small_order, "checked_scalar": checked}


def main():
    if not build_ref(REF):
        sys.exit("reference not available")
    ref = RefLib()
    with open(os.path.join(OUT, "poh_332.json"), "w") as f:
        json.dump(poh_fixture(), f, indent=0)
    with open(os.path.join(OUT, "ed25519_ref.json"), "w") as f:
        json.dump(ed25519_fixture(ref), f, indent=0)
    print("wrote", os.listdir(OUT))


if __name__ == "__main__":
    main()
