#!/usr/bin/env python3
"""Full-size expected outputs of the five benchmark workloads, as digests.

The workloads (solana-perf-libs_gb300/workloads.py, seeded) are too large to
commit as vectors, so this script runs them once on the CPU and writes
SHA-256 digests of their inputs and expected outputs to config_digests.json:

  verify_1024     1024 packets [sig][pk][64-B msg], 10% bit-flipped (seed 1)
  poh_uniform     4096 entries x 12500 hashes (seed 2)
  ragged_sigs     64 ragged verify batches + their 128-packet signing jobs
                  (seed 3): 100,738 verifies and 100,738 signatures
  poh_ragged      16384 entries, num_hashes log-uniform in 1..1e6 (seed 4),
                  3% of the expected hashes corrupted (seed 44)

Expected outputs come from the reference's own host code, compiled from its
sources into oracle/_ref by oracle/ref.mk: keypairs from
ed25519_create_keypair (src/cuda-ecc-ed25519/keypair.cu:6-16), signatures
from ed25519_sign (sign.cu:40-46), verdicts from ed25519_verify
(verify.cu:154-174), PoH from its host SHA-256 chained as poh_verify_kernel
chains it (src/cuda-poh-verify/poh_verify.cu:12-27).  Every figure is
checked against the CPU oracle (oracle/crypt_oracle.c) before it is written.

Needs the reference tree (REF_ROOT, default /root/reference) on an x86_64
host; about two minutes on 8 cores.  Run from the repository root:
    python3 tests/golden/make_config_digests.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "solana-perf-libs_gb300"))

import workloads  # noqa: E402
from oracle.oracle import RefLib, build_ref, get_oracle  # noqa: E402

REF = os.environ.get("REF_ROOT", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "config_digests.json")
THREADS = os.cpu_count() or 1
POH_CORRUPT_SEED = 44


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


class RefCalls:
    """The reference's single-item host calls, spread over host threads (ctypes
    releases the interpreter lock during each call)."""

    def __init__(self, ref: RefLib):
        self.ref = ref
        self.pool = ThreadPoolExecutor(THREADS)

    def keypairs(self, seeds):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint8).reshape(-1, 32)
        res = list(self.pool.map(lambda s: self.ref.create_keypair(bytes(s)), seeds))
        pk = np.frombuffer(b"".join(r[0] for r in res), dtype=np.uint8).reshape(-1, 32).copy()
        sk = np.frombuffer(b"".join(r[1] for r in res), dtype=np.uint8).reshape(-1, 64).copy()
        return pk, sk

    def _items(self, sp):
        flat = sp.concatenated()
        n = sp.total_signatures
        ml, ko, so, mo = (np.asarray(a, dtype=np.int64) for a in
                          (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets))
        return [(bytes(flat[so[i]:so[i] + 64]), bytes(flat[mo[i]:mo[i] + ml[i]]), bytes(flat[ko[i]:ko[i] + 32]))
                for i in range(n)]

    def sign(self, sp):
        """sign_many over a SigPackets: the key-offset slot holds the 64-byte
        expanded secret key (the reference's sign_many layout)."""
        items = self._items(sp)
        sigs = list(self.pool.map(lambda t: self.ref.sign(t[1], t[2], t[0]), items))
        return np.frombuffer(b"".join(sigs), dtype=np.uint8).reshape(-1, 64).copy()

    def verify(self, sp):
        items = self._items(sp)
        return np.array(list(self.pool.map(lambda t: self.ref.verify(*t), items)), dtype=np.uint8)

    def poh(self, hashes, counts):
        rows = [bytes(r) for r in np.asarray(hashes, dtype=np.uint8).reshape(-1, 32)]
        order = np.argsort(-np.asarray(counts, dtype=np.int64), kind="stable")     # longest first
        out = [None] * len(rows)

        def run(i):
            out[i] = self.ref.poh_chain(rows[i], int(counts[i]))
        list(self.pool.map(run, order))
        return np.frombuffer(b"".join(out), dtype=np.uint8).reshape(-1, 32).copy()


def verify_1024(rc: RefCalls, o):
    sp, corrupted = workloads.verify_uniform(rc.keypairs, rc.sign, n=1024, seed=1)
    v = rc.verify(sp)
    assert np.array_equal(v, o.verify_packets(sp, THREADS))
    assert np.array_equal(v.astype(bool), ~corrupted)
    return {"workload": "workloads.verify_uniform(n=1024, seed=1)", "signatures": 1024,
            "input_sha256": digest(sp.concatenated()), "verdicts_sha256": digest(v),
            "accepted": int(v.sum())}


def poh_uniform(rc: RefCalls, o):
    h, c = workloads.poh_uniform(4096, 12500, seed=2)
    f = rc.poh(h, c)
    assert np.array_equal(f, o.poh_verify_many(h, c, THREADS))
    return {"workload": "workloads.poh_uniform(4096, 12500, seed=2)", "entries": 4096,
            "input_sha256": digest(h, c), "final_sha256": digest(f)}


def ragged_sigs(rc: RefCalls, o):
    rs = workloads.ragged_sigs(rc.keypairs, rc.sign, seed=3)
    verdicts = [rc.verify(sp) for sp in rs.verify]
    sigs = [rc.sign(sp) for sp in rs.sign]
    for sp, v in zip(rs.verify, verdicts):
        assert np.array_equal(v, o.verify_packets(sp, THREADS))
    for sp, s in zip(rs.sign, sigs):
        assert np.array_equal(s, o.sign_packets(sp, THREADS))
    cls = np.concatenate(rs.classes)
    ver = np.concatenate(verdicts)
    per_class = {name: {"count": int((cls == k).sum()), "accepted": int(ver[cls == k].sum())}
                 for k, name in enumerate(("valid", "s_ge_l", "small_order_a", "small_order_r", "undecodable_a",
                                           "flipped_message"))}
    return {"workload": "workloads.ragged_sigs(seed=3)", "verify_batches": len(rs.verify),
            "sign_jobs": len(rs.sign), "verify_signatures": int(len(ver)),
            "sign_signatures": int(sum(len(s) for s in sigs)),
            "verify_input_sha256": digest(*[sp.concatenated() for sp in rs.verify]),
            "verify_offsets_sha256": digest(*[np.asarray(a, dtype=np.uint32) for sp in rs.verify for a in
                                              (sp.message_lens, sp.public_key_offsets, sp.signature_offsets,
                                               sp.message_start_offsets)]),
            "verdicts_sha256": digest(ver), "signatures_sha256": digest(*sigs),
            "accepted": int(ver.sum()), "per_class": per_class}


def poh_ragged(rc: RefCalls, o):
    h, c = workloads.poh_ragged(16384, 1_000_000, seed=4)
    f = rc.poh(h, c)
    assert np.array_equal(f, o.poh_verify_many(h, c, THREADS))
    exp, mask = workloads.corrupt_expected(f, 0.03, POH_CORRUPT_SEED)
    flags = np.all(f == exp, axis=1).astype(np.uint8)
    assert np.array_equal(flags.astype(bool), ~mask)
    return {"workload": "workloads.poh_ragged(16384, 1e6, seed=4)", "entries": 16384,
            "total_hashes": int(c.sum()), "longest_chain": int(c.max()),
            "input_sha256": digest(h, c), "final_sha256": digest(f),
            "corrupt_seed": POH_CORRUPT_SEED, "corrupted_expected_sha256": digest(exp),
            "flags_sha256": digest(flags), "passing": int(flags.sum())}


def main():
    if not build_ref(REF):
        sys.exit("reference not available")
    rc = RefCalls(RefLib())
    o = get_oracle()
    res = {"source": "reference host code (oracle/_ref), cross-checked against the CPU oracle",
           "digest": "sha256 over the concatenated raw bytes (uint8 verdicts, 64-byte signatures, "
                     "32-byte hashes, uint32 offsets, uint64 counts)"}
    for name, fn in (("verify_1024", verify_1024), ("poh_uniform", poh_uniform), ("ragged_sigs", ragged_sigs),
                     ("poh_ragged", poh_ragged)):
        t = time.time()
        res[name] = fn(rc, o)
        print(f"{name}: {time.time() - t:.1f} s", flush=True)
    with open(OUT, "w") as f:
        json.dump(res, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
