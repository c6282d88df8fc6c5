"""The verify forms -- four lanes per signature (verify_quad.cuh), three
warps per eight signatures with half-size scalars (verify_trio.cuh), and one lane
per signature with a 4- or 5-bit window of h -- against the golden
verdicts, the oracle and the one-thread kernel, with the cases that
exercise their own final checks (R decoded and compared projectively, or
[d]([S]B - [h]A - R) tested against the neutral point, instead of encode +
byte compare): R with its sign bit flipped, every non-canonical y >= p,
undecodable R, R set to other valid points and to every small-order
encoding, keys and nonces with small-order components, partial quads,
trios and warps."""
import numpy as np
import pytest

import workloads
from conftest import nthreads
from test_gpu_verify import pack_items

pytestmark = pytest.mark.gpu

P = 2 ** 255 - 19


def run_form(lib, sp, form):
    torch = pytest.importorskip("torch")
    d = torch.from_numpy(sp.concatenated().copy()).cuda()
    arrs = [torch.from_numpy(np.asarray(a, dtype=np.int64).astype(np.int32)).cuda()
            for a in (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)]
    out = torch.full((sp.total_signatures,), 7, dtype=torch.uint8, device="cuda")
    lib.verify_device_form(d, *arrs, out, form, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def ALL_FORMS(lib):
    return (lib.VERIFY_SINGLE, lib.VERIFY_QUAD, lib.VERIFY_SINGLE_W4, lib.VERIFY_SINGLE_W5, lib.VERIFY_TRIO,
            lib.VERIFY_STAGED, lib.VERIFY_HALF)


def both_forms(lib, oracle, sp):
    """Every verify form (one lane with 4- and 5-bit windows, four lanes,
    three warps per eight) against the oracle."""
    exp = oracle.verify_packets(sp, nthreads())
    for form in ALL_FORMS(lib):
        assert np.array_equal(run_form(lib, sp, form), exp), form
    return exp


def test_quad_golden(lib, golden_ed):
    cases = golden_ed["verify"]
    items = [(bytes.fromhex(c["sig"]), bytes.fromhex(c["msg"]), bytes.fromhex(c["pk"])) for c in cases]
    sp = pack_items(items, gap_seed=5)
    exp = np.array([c["valid"] for c in cases], dtype=np.uint8)
    for form in ALL_FORMS(lib):
        got = run_form(lib, sp, form)
        bad = [cases[i]["kind"] for i in np.nonzero(got != exp)[0]]
        assert not bad, (form, bad)


def test_quad_uniform_and_ragged(lib, oracle):
    sp, corrupted = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=1024, seed=51)
    exp = both_forms(lib, oracle, sp)
    assert np.array_equal(exp.astype(bool), ~corrupted)
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=4, total_packet_cap=300,
                               seed=52)
    for sp in rs.verify:
        both_forms(lib, oracle, sp)


def _valid_items(oracle, n, seed, msg_len=None):
    rng = np.random.default_rng(seed)
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    items = []
    for i in range(n):
        m = int(rng.integers(0, 300)) if msg_len is None else msg_len
        msg = bytes(rng.integers(0, 256, m, dtype=np.uint8).tolist())
        items.append((oracle.sign(msg, bytes(pk[i]), bytes(sk[i])), msg, bytes(pk[i])))
    return items, rng


def test_quad_r_variants(lib, oracle):
    items, rng = _valid_items(oracle, 64, 53)
    so = workloads.small_order_encodings()
    cases = list(items)
    for sig, msg, pk in items:
        s = bytearray(sig)
        s[31] ^= 0x80                                     # R's sign bit
        cases.append((bytes(s), msg, pk))
        s = bytearray(sig)
        s[:32] = rng.integers(0, 256, 32, dtype=np.uint8).tobytes()     # random R (mostly undecodable)
        cases.append((bytes(s), msg, pk))
        s = bytearray(sig)
        s[:32] = items[int(rng.integers(0, len(items)))][2]             # another valid point
        cases.append((bytes(s), msg, pk))
    sig, msg, pk = items[0]
    for k in range(19):                                   # y = p + k, both sign bits
        for sign in (0, 1):
            y = P + k
            enc = bytearray(y.to_bytes(32, "little"))
            enc[31] |= sign << 7
            cases.append((bytes(enc) + sig[32:], msg, pk))
    for enc in so:                                        # every small-order R and A
        cases.append((enc + sig[32:], msg, pk))
        cases.append((sig, msg, enc))
    sp = pack_items(cases, gap_seed=6)
    exp = both_forms(lib, oracle, sp)
    assert exp[:64].all() and not exp[64:64 + 3 * 64].all()


def test_quad_message_lengths_and_random(lib, oracle):
    rng2 = np.random.default_rng(55)
    seeds = rng2.integers(0, 256, (1, 32), dtype=np.uint8)
    pkk, skk = oracle.create_keypairs(seeds)
    cases = []
    for m in range(0, 260):
        msg = bytes(rng2.integers(0, 256, m, dtype=np.uint8).tolist())
        sig = oracle.sign(msg, bytes(pkk[0]), bytes(skk[0]))
        cases.append((sig, msg, bytes(pkk[0])))
        bad = bytearray(sig)
        bad[int(rng2.integers(0, 64))] ^= 1 << int(rng2.integers(0, 8))
        cases.append((bytes(bad), msg, bytes(pkk[0])))
    for i in range(600):
        sig = bytearray(rng2.integers(0, 256, 64, dtype=np.uint8).tolist())
        if i % 2:
            sig[63] &= 0x0F
        cases.append((bytes(sig), b"x" * (i % 50), rng2.integers(0, 256, 32, dtype=np.uint8).tobytes()))
    both_forms(lib, oracle, pack_items(cases, gap_seed=7))


def mixed_order_items(n=160, seed=57):
    """(signature, message, public key) items with A = aB + T and
    R = rB + T' for small-order T, T' (every order 1..8), signed with the
    discrete logs: S = r + h a mod L.  The reference's cofactorless check
    accepts exactly when [h]T = -T' (e.g. T' neutral and 8 | h for T of
    order 8), so both verdicts occur."""
    import hashlib
    import ed25519_math as E
    by = 4 * pow(5, E.P - 2, E.P) % E.P
    B = (E.recover_x(by, 0), by)
    tors = E.torsion_points()
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(n):
        a = int.from_bytes(rng.bytes(32), "little") % E.L
        r = int.from_bytes(rng.bytes(32), "little") % E.L
        ta = tors[k % len(tors)]
        tr = tors[(k // len(tors)) % len(tors)] if k % 3 == 0 else (0, 1)
        A = E.encode(E.add(E.mul(a, B), ta))
        R = E.encode(E.add(E.mul(r, B), tr))
        msg = rng.bytes(int(rng.integers(0, 100)))
        h = int.from_bytes(hashlib.sha512(R + A + msg).digest(), "little") % E.L
        S = (r + h * a) % E.L
        cases.append((R + S.to_bytes(32, "little"), msg, A))
    return cases


def test_mixed_order_keys_and_nonces(lib, oracle):
    """Every form agrees with the oracle on keys and nonces with small-order
    components (the half-size-scalar forms: their modulus 8L keeps the
    small-order part of [h]A exact)."""
    cases = mixed_order_items()
    exp = both_forms(lib, oracle, pack_items(cases, gap_seed=9))
    assert 0 < int(exp.sum()) < len(cases)


@pytest.mark.parametrize("n", [1, 3, 7, 8, 9, 33, 257, 1217, 2500])
def test_quad_partial_quads_and_warps(lib, oracle, n):
    items, _ = _valid_items(oracle, n, 56 + n, msg_len=40)
    exp = both_forms(lib, oracle, pack_items(items, gap_seed=8))
    assert exp.all()


def test_verify_form_rejects_bad_form(lib):
    torch = pytest.importorskip("torch")
    z = torch.zeros(4, dtype=torch.int32, device="cuda")
    out = torch.zeros(4, dtype=torch.uint8, device="cuda")
    with pytest.raises(RuntimeError):
        lib.verify_device_form(torch.zeros(256, dtype=torch.uint8, device="cuda"), z, z, z, z, out, 7)


def test_half_scalars_chosen_h(lib):
    """The half-size scalar search of the three-warp form on chosen h (which no
    signature can choose, h being a hash): c = d h (mod 8L) with d odd and
    positive for every h; about 128-bit |c| and d for random h; the
    full-length pair (h, 1) for h next to a fraction with a small even
    denominator, where no short pair has d odd."""
    torch = pytest.importorskip("torch")
    L = 2 ** 252 + 27742317777372353535851937790883648493
    M = 8 * L
    rng = np.random.default_rng(58)
    hs = [0, 1, 2, 3, 5, L - 1, L - 2, (L - 1) // 2, L // 3, L // 7, 2 ** 252 - 1, 2 ** 200, 2 ** 128,
          2 ** 127 + 1, (1 << 250) + 12345]
    hs += [int.from_bytes(rng.bytes(32), "little") % L for _ in range(4000)]
    hs += [int.from_bytes(rng.bytes(32), "little") >> int(rng.integers(1, 250)) for _ in range(500)]
    words = np.array([[(h >> (32 * k)) & 0xffffffff for k in range(8)] for h in hs], dtype=np.uint32)
    dh = torch.from_numpy(words.view(np.int32)).cuda()
    out = torch.zeros((len(hs), 18), dtype=torch.int32, device="cuda")
    lib.half_scalars_device(dh, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    o = out.cpu().numpy().view(np.uint32)
    longest = 0
    for k, h in enumerate(hs):
        c = sum(int(o[k, j]) << (32 * j) for j in range(8))
        d = sum(int(o[k, 9 + j]) << (32 * j) for j in range(8))
        if o[k, 8]:
            c = -c
        assert (c - d * h) % M == 0 and d % 2 == 1 and d > 0, k
        assert o[k, 17] < 768, k
        if 15 <= k < 4015:
            longest = max(longest, abs(c).bit_length(), d.bit_length())
    assert longest <= 150
    assert sum(int(o[5, 9 + j]) << (32 * j) for j in range(8)) == 1      # h = L - 1: the full-length pair
