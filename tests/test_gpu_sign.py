"""Ed25519 signing and keypair derivation on the GPU: byte-identical to the
reference's golden keys/signatures and to the CPU oracle."""
import numpy as np
import pytest

import workloads
from cuda_crypt import SigPackets
from conftest import nthreads

pytestmark = pytest.mark.gpu


def test_keypairs_golden(lib, golden_ed):
    seeds = np.array([list(bytes.fromhex(k["seed"])) for k in golden_ed["keys"]], dtype=np.uint8)
    pk, sk = lib.create_keypairs(seeds)
    for i, k in enumerate(golden_ed["keys"]):
        assert bytes(pk[i]).hex() == k["pk"]
        assert bytes(sk[i]).hex() == k["sk"]
    p1, s1 = lib.create_keypair(bytes.fromhex(golden_ed["keys"][0]["seed"]))
    assert p1.hex() == golden_ed["keys"][0]["pk"] and s1.hex() == golden_ed["keys"][0]["sk"]


def test_sign_golden(lib, golden_ed):
    keys = {k["pk"]: k for k in golden_ed["keys"]}
    for c in golden_ed["verify"]:
        if c["kind"] != "valid":
            continue
        k = keys[c["pk"]]
        assert lib.sign(bytes.fromhex(c["msg"]), bytes.fromhex(k["pk"]), bytes.fromhex(k["sk"])).hex() == c["sig"]


def _sign_items(items):
    """items: (msg, pk, sk) -> SigPackets laid out [sk][pk][msg] per packet."""
    maxlen = max(len(m) for m, _, _ in items)
    stride = 3 + 64 + 32 + maxlen
    n = len(items)
    pkt = np.zeros((n, stride), dtype=np.uint8)
    idx = np.arange(n, dtype=np.uint32)
    lens = np.zeros(n, dtype=np.uint32)
    for i, (m, pk, sk) in enumerate(items):
        pkt[i, 3:67] = np.frombuffer(sk, dtype=np.uint8)
        pkt[i, 67:99] = np.frombuffer(pk, dtype=np.uint8)
        if m:
            pkt[i, 99:99 + len(m)] = np.frombuffer(m, dtype=np.uint8)
        lens[i] = len(m)
    return SigPackets([pkt.ravel()], stride, lens, idx * stride + 67, idx * stride + 3, idx * stride + 99)


def test_sign_many_vs_oracle(lib, oracle):
    rng = np.random.default_rng(51)
    n = 700
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    items = []
    for i in range(n):
        m = bytes(rng.integers(0, 256, int(rng.integers(0, 300)), dtype=np.uint8).tolist())
        key = bytes(sk[i]) if i % 5 else bytes(rng.integers(0, 256, 64, dtype=np.uint8).tolist())  # unclamped too
        items.append((m, bytes(pk[i]), key))
    sp = _sign_items(items)
    assert np.array_equal(lib.sign_many(sp), oracle.sign_packets(sp, nthreads()))
    assert np.array_equal(lib.sign_many(sp, use_non_default_stream=0), oracle.sign_packets(sp, nthreads()))


def test_sign_ragged_batches(lib, oracle):
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=3, total_packet_cap=300,
                               seed=52)
    for sp in rs.sign:
        assert np.array_equal(lib.sign_many(sp), oracle.sign_packets(sp, nthreads()))


def test_sign_then_verify_roundtrip(lib):
    sp, corrupted = workloads.verify_uniform(lib.create_keypairs, lib.sign_many, n=256, flip_frac=0.0, seed=53)
    assert lib.verify_many(sp).all()


def test_sign_device_form(lib, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(54)
    n = 200
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    items = [(bytes(rng.integers(0, 256, 40, dtype=np.uint8).tolist()), bytes(pk[i]), bytes(sk[i])) for i in range(n)]
    sp = _sign_items(items)
    exp = oracle.sign_packets(sp, nthreads())
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    out = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
    lib.sign_device(dev(sp.concatenated()), *(dev(a.astype(np.int32)) for a in
                    (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)),
                    out, torch.cuda.current_stream().cuda_stream)
    seeds = dev(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    dpk = torch.zeros((n, 32), dtype=torch.uint8, device="cuda")
    dsk = torch.zeros((n, 64), dtype=torch.uint8, device="cuda")
    lib.keypair_device(seeds, dpk, dsk, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), exp)
    epk, esk = oracle.create_keypairs(seeds.cpu().numpy())
    assert np.array_equal(dpk.cpu().numpy(), epk) and np.array_equal(dsk.cpu().numpy(), esk)


def test_sign_many_shared_inversion(lib, oracle):
    """From 80,000 signatures a launch shares one field inversion per block
    (sign.cu): 82,000 signatures, the last block partial, equal the oracle's;
    with a few items' offsets out of range, those signatures are zero and
    every other one in their blocks is unchanged."""
    rng = np.random.default_rng(55)
    n = 82000
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    lens = rng.integers(0, 65, n)
    items = [(bytes(rng.integers(0, 256, int(lens[i]), dtype=np.uint8).tolist()), bytes(pk[i]),
              bytes(sk[i]) if i % 7 else bytes(rng.integers(0, 256, 64, dtype=np.uint8).tolist()))
             for i in range(n)]
    sp = _sign_items(items)
    got = lib.sign_many(sp)
    assert np.array_equal(got, oracle.sign_packets(sp, nthreads()))
    bad = np.array([5, 130, n - 1])
    mso = sp.message_start_offsets.copy()
    mso[bad] = len(sp.concatenated()) + 1
    sp2 = SigPackets(sp.batches, sp.message_size, sp.message_lens, sp.public_key_offsets, sp.signature_offsets, mso)
    got2 = lib.sign_many(sp2)
    keep = np.setdiff1d(np.arange(n), bad)
    assert not got2[bad].any() and np.array_equal(got2[keep], got[keep])
