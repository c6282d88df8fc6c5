"""Ed25519 batch verification on the GPU against the reference's golden
verdicts (tests/golden/ed25519_ref.json) and the CPU oracle: identical
per-signature verdicts, quirks included."""
import numpy as np
import pytest

import workloads
from cuda_crypt import SigPackets
from conftest import nthreads

pytestmark = pytest.mark.gpu


def pack_items(items, gap_seed=0, elems_split=1):
    """items: list of (sig, msg, pk) -> SigPackets with one packet per item,
    laid out [gap][sig][pk][msg] at unaligned offsets."""
    rng = np.random.default_rng(gap_seed)
    maxlen = max(len(m) for _, m, _ in items) if items else 0
    stride = 16 + 64 + 32 + maxlen
    n = len(items)
    pkt = np.zeros((n, stride), dtype=np.uint8)
    lens = np.zeros(n, dtype=np.uint32)
    so = np.zeros(n, dtype=np.uint32)
    po = np.zeros(n, dtype=np.uint32)
    mo = np.zeros(n, dtype=np.uint32)
    for i, (sig, msg, pk) in enumerate(items):
        g = int(rng.integers(0, 16))
        pkt[i, g:g + 64] = np.frombuffer(sig, dtype=np.uint8)
        pkt[i, g + 64:g + 96] = np.frombuffer(pk, dtype=np.uint8)
        if msg:
            pkt[i, g + 96:g + 96 + len(msg)] = np.frombuffer(msg, dtype=np.uint8)
        lens[i] = len(msg)
        so[i], po[i], mo[i] = i * stride + g, i * stride + g + 64, i * stride + g + 96
    flat = pkt.ravel()
    cuts = np.linspace(0, n, elems_split + 1).astype(int)
    batches = [flat[cuts[k] * stride:cuts[k + 1] * stride].copy() for k in range(elems_split)]
    return SigPackets(batches, stride, lens, po, so, mo)


def test_verify_golden(lib, golden_ed):
    cases = golden_ed["verify"]
    items = [(bytes.fromhex(c["sig"]), bytes.fromhex(c["msg"]), bytes.fromhex(c["pk"])) for c in cases]
    sp = pack_items(items, gap_seed=1, elems_split=3)
    got = lib.verify_many(sp)
    exp = np.array([c["valid"] for c in cases], dtype=np.uint8)
    bad = [cases[i]["kind"] for i in np.nonzero(got != exp)[0]]
    assert not bad, bad


def test_verify_uniform_full_size(lib, oracle):
    """1024 packets [sig][pk][64-B msg], 10% with one flipped bit."""
    sp, corrupted = workloads.verify_uniform(lib.create_keypairs, lib.sign_many)
    exp = oracle.verify_packets(sp, nthreads())
    got = lib.verify_many(sp)
    assert np.array_equal(got, exp)
    assert np.array_equal(got.astype(bool), ~corrupted)


def test_verify_ragged_subset(lib, oracle):
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=6, total_packet_cap=400,
                               seed=31)
    for sp, cls in zip(rs.verify, rs.classes):
        exp = oracle.verify_packets(sp, nthreads())
        got = lib.verify_many(sp)
        assert np.array_equal(got, exp)
        # every adversarial class is rejected; valid ones pass
        assert np.all(got[cls == workloads.CLASS_VALID] == 1)
        assert np.all(got[(cls != workloads.CLASS_VALID) & (cls != workloads.CLASS_SMALL_A)
                          & (cls != workloads.CLASS_SMALL_R)] == 0)


def test_verify_message_lengths(lib, oracle):
    """Every length across the SHA-512 block boundaries (R||A||M = 64 + m)."""
    rng = np.random.default_rng(41)
    seeds = rng.integers(0, 256, (1, 32), dtype=np.uint8)
    pk, sk = oracle.create_keypairs(seeds)
    pk, sk = bytes(pk[0]), bytes(sk[0])
    items = []
    for m in range(0, 400):
        msg = bytes(rng.integers(0, 256, m, dtype=np.uint8).tolist())
        sig = oracle.sign(msg, pk, sk)
        items.append((sig, msg, pk))
        bad = bytearray(sig)
        bad[int(rng.integers(0, 64))] ^= 1 << int(rng.integers(0, 8))
        items.append((bytes(bad), msg, pk))
    sp = pack_items(items, gap_seed=2)
    exp = oracle.verify_packets(sp, nthreads())
    got = lib.verify_many(sp)
    assert np.array_equal(got, exp)
    assert got[0::2].all()


def test_verify_random_inputs(lib, oracle):
    """Random bytes everywhere: almost all invalid, but every verdict must
    match (exercises decode failures and S checks)."""
    rng = np.random.default_rng(42)
    items = []
    for i in range(2000):
        sig = bytearray(rng.integers(0, 256, 64, dtype=np.uint8).tolist())
        if i % 2:
            sig[63] &= 0x0F
        items.append((bytes(sig), bytes(rng.integers(0, 256, int(rng.integers(0, 100)), dtype=np.uint8).tolist()),
                      bytes(rng.integers(0, 256, 32, dtype=np.uint8).tolist())))
    sp = pack_items(items, gap_seed=3)
    assert np.array_equal(lib.verify_many(sp), oracle.verify_packets(sp, nthreads()))


def test_verify_empty_calls_leave_out_untouched(lib):
    sp = pack_items([(bytes(64), b"", bytes(32))])
    out = np.full(1, 7, dtype=np.uint8)
    import ctypes
    from cuda_crypt import _p, _u8p, _u32p
    arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
            (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)]
    elems = lib._elems(sp.batches, sp.message_size)
    # total_packets == 0
    lib.lib.ed25519_verify_many(elems, 1, sp.message_size, 0, 1, *[_p(a, _u32p) for a in arrs], _p(out, _u8p), 1)
    assert out[0] == 7
    # total_signatures == 0
    lib.lib.ed25519_verify_many(elems, 1, sp.message_size, 1, 0, *[_p(a, _u32p) for a in arrs], _p(out, _u8p), 1)
    assert out[0] == 7


def test_verify_out_of_range_offsets_rejected(lib, oracle):
    rng = np.random.default_rng(43)
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (1, 32), dtype=np.uint8))
    msg = b"abcd1234"
    sig = oracle.sign(msg, bytes(pk[0]), bytes(sk[0]))
    sp = pack_items([(sig, msg, bytes(pk[0]))] * 4)
    total = sum(len(b) for b in sp.batches)
    sp.signature_offsets = sp.signature_offsets.copy()
    sp.public_key_offsets = sp.public_key_offsets.copy()
    sp.message_lens = sp.message_lens.copy()
    sp.signature_offsets[1] = total - 10
    sp.public_key_offsets[2] = 0xFFFFFFF0
    sp.message_lens[3] = 0xFFFFFFFF
    got = lib.verify_many(sp)
    assert list(got) == [1, 0, 0, 0]


def test_verify_default_stream_and_pinned(lib, oracle):
    sp, _ = workloads.verify_uniform(lib.create_keypairs, lib.sign_many, n=300, seed=44)
    exp = oracle.verify_packets(sp, nthreads())
    assert np.array_equal(lib.verify_many(sp, use_non_default_stream=0), exp)
    buf = sp.batches[0]
    assert lib.host_register(buf) == 0
    try:
        assert np.array_equal(lib.verify_many(sp), exp)
    finally:
        assert lib.host_unregister(buf) == 0


def test_single_item_forms(lib, golden_ed):
    for c in golden_ed["verify"][:120]:
        assert lib.verify(bytes.fromhex(c["sig"]), bytes.fromhex(c["msg"]), bytes.fromhex(c["pk"])) == c["valid"]
    for c in golden_ed["small_order"]:
        assert lib.check_packed_ge_small_order(bytes.fromhex(c["point"])) == c["result"], c
    for c in golden_ed["checked_scalar"]:
        assert lib.get_checked_scalar(bytes.fromhex(c["scalar"])) == c["result"], c


def test_verify_device_form(lib, oracle):
    torch = pytest.importorskip("torch")
    sp, _ = workloads.verify_uniform(lib.create_keypairs, lib.sign_many, n=500, seed=45)
    exp = oracle.verify_packets(sp, nthreads())
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pk = dev(sp.concatenated())
    lens, po, so, mo = (dev(a.astype(np.int32)) for a in
                        (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets))
    out = torch.zeros(len(exp), dtype=torch.uint8, device="cuda")
    lib.verify_device(pk, lens, po, so, mo, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), exp)


@pytest.mark.parametrize("register", [False, True])
def test_verify_and_sign_with_empty_runs(lib, oracle, register):
    """gpu_Elems runs with empty ones between them (num = 0), from pageable
    buffers and from buffers page-locked with cuda_host_register (copied run
    by run straight from the caller's memory)."""
    from test_gpu_sign import _sign_items
    rng = np.random.default_rng(47)
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (90, 32), dtype=np.uint8))
    items = []
    for i in range(90):
        msg = rng.bytes(int(rng.integers(0, 200)))
        sig = oracle.sign(msg, bytes(pk[i]), bytes(sk[i]))
        if i % 7 == 3:
            sig = sig[:5] + bytes([sig[5] ^ 1]) + sig[6:]
        items.append((sig, msg, bytes(pk[i])))
    sp = pack_items(items, gap_seed=12, elems_split=3)
    empty = np.zeros(0, dtype=np.uint8)
    sp.batches = [empty, sp.batches[0], empty, empty, sp.batches[1], sp.batches[2], empty]
    ssp = _sign_items([(rng.bytes(int(rng.integers(0, 150))), bytes(pk[i]), bytes(sk[i])) for i in range(40)])
    flat = ssp.batches[0]
    cut = (len(flat) // ssp.message_size // 2) * ssp.message_size
    ssp.batches = [flat[:cut].copy(), empty, flat[cut:].copy()]
    regs = [b for b in sp.batches + ssp.batches if b.nbytes] if register else []
    for b in regs:
        assert lib.host_register(b) == 0
    try:
        assert np.array_equal(lib.verify_many(sp), oracle.verify_packets(sp, nthreads()))
        assert np.array_equal(lib.sign_many(ssp), oracle.sign_packets(ssp, nthreads()))
    finally:
        for b in regs:
            lib.host_unregister(b)
