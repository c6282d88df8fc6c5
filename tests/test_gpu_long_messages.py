"""Messages far longer than a packet: the reference takes any 32-bit
message length, so R||A||M runs through many SHA-512 blocks.  Lengths just
past the 1,232-byte packet limit up to ~200 KB, short ones beside them in
one launch (lanes with very different block counts), against the oracle in
every verify form, in sign_many, and in one mixed batched launch."""
import numpy as np
import pytest

from conftest import nthreads
from cuda_crypt import JOB_SIGN, JOB_VERIFY
from test_gpu_sign import _sign_items
from test_gpu_verify import pack_items
from test_gpu_verify_quad import run_form

pytestmark = pytest.mark.gpu

LENGTHS = [0, 17, 1232, 1233, 2047, 2048, 4103, 16387, 65647, 200003]


def _keys(oracle, n, seed):
    rng = np.random.default_rng(seed)
    pk, sk = oracle.create_keypairs(rng.integers(0, 256, (n, 32), dtype=np.uint8))
    return rng, [bytes(p) for p in pk], [bytes(s) for s in sk]


def _verify_items(oracle, seed):
    """Each length signed, then the same signature over the message with its
    last byte changed, and with a byte in the middle changed."""
    rng, pks, sks = _keys(oracle, len(LENGTHS), seed)
    items = []
    for k, m in enumerate(LENGTHS):
        msg = rng.bytes(m)
        sig = oracle.sign(msg, pks[k], sks[k])
        items.append((sig, msg, pks[k]))
        if m:
            for pos in (m - 1, m // 2):
                bad = bytearray(msg)
                bad[pos] ^= 0x40
                items.append((sig, bytes(bad), pks[k]))
    return items


def test_verify_long_messages_every_form(lib, oracle):
    items = _verify_items(oracle, 401)
    sp = pack_items(items, gap_seed=9, elems_split=3)     # 5.6 MB in three runs: the parallel staging copy
    exp = oracle.verify_packets(sp, nthreads())
    assert exp.sum() == len(LENGTHS)                       # the signed messages, none of the altered ones
    assert np.array_equal(lib.verify_many(sp), exp)
    for form in (lib.VERIFY_SINGLE, lib.VERIFY_QUAD, lib.VERIFY_SINGLE_W4, lib.VERIFY_SINGLE_W5):
        assert np.array_equal(run_form(lib, sp, form), exp), form


def test_sign_long_messages(lib, oracle):
    rng, pks, sks = _keys(oracle, len(LENGTHS), 402)
    sp = _sign_items([(rng.bytes(m), pks[k], sks[k]) for k, m in enumerate(LENGTHS)])
    assert np.array_equal(lib.sign_many(sp), oracle.sign_packets(sp, nthreads()))


def test_batched_launch_long_and_short(lib, oracle):
    """One persistent launch: a long-message verify job and sign job beside
    short-message ones."""
    items = _verify_items(oracle, 403)
    v_long = pack_items(items, gap_seed=10)
    v_short = pack_items(items[:3], gap_seed=11)
    rng, pks, sks = _keys(oracle, len(LENGTHS), 404)
    s_long = _sign_items([(rng.bytes(m), pks[k], sks[k]) for k, m in enumerate(LENGTHS)])
    s_short = _sign_items([(rng.bytes(20), pks[k], sks[k]) for k in range(4)])
    jobs = [(v_long, JOB_VERIFY), (s_short, JOB_SIGN), (v_short, JOB_VERIFY), (s_long, JOB_SIGN)]
    outs = lib.ed25519_batch(jobs)
    assert np.array_equal(outs[0], oracle.verify_packets(v_long, nthreads()))
    assert np.array_equal(outs[1], oracle.sign_packets(s_short, nthreads()))
    assert np.array_equal(outs[2], oracle.verify_packets(v_short, nthreads()))
    assert np.array_equal(outs[3], oracle.sign_packets(s_long, nthreads()))
