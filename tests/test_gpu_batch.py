"""Ragged batches in one persistent launch (gb300_ed25519_batch,
gb300_poh_verify_batch and their device forms): identical results to the
per-call entry points and to the CPU oracle, including repeated calls that
replay a captured CUDA graph and calls that change the batch shape."""
import numpy as np
import pytest

import workloads
from cuda_crypt import JOB_SIGN, JOB_VERIFY
from conftest import nthreads

pytestmark = pytest.mark.gpu


def test_poh_batch_ragged(lib, oracle):
    h, cnt = workloads.poh_ragged(n=3000, max_hashes=20000, seed=61)
    cnt[:7] = [0, 1, 2, 0, 20000, 31, 32]
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    for rep in range(3):                      # first call captures, later calls replay the graph
        buf = h.ravel().copy()
        assert lib.poh_verify_batch(buf, cnt) == 0
        assert np.array_equal(buf.reshape(-1, 32), exp), rep
    # another shape
    buf = h[:1234].ravel().copy()
    assert lib.poh_verify_batch(buf, cnt[:1234]) == 0
    assert np.array_equal(buf.reshape(-1, 32), exp[:1234])


def test_poh_batch_matches_plain_on_many_chains(lib):
    """More chains than resident lanes (lanes take several chains each)."""
    rng = np.random.default_rng(62)
    n = 40000
    h = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    cnt = rng.integers(0, 300, n).astype(np.uint64)
    a = h.ravel().copy()
    b = a.copy()
    assert lib.poh_verify_many(a, cnt) == 0
    assert lib.poh_verify_batch(b, cnt) == 0
    assert np.array_equal(a, b)


def test_poh_batch_device(lib, oracle):
    torch = pytest.importorskip("torch")
    h, cnt = workloads.poh_ragged(n=2000, max_hashes=5000, seed=63)
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    dh = torch.from_numpy(h.copy()).cuda()
    dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
    ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
    lib.poh_verify_batch_device(dh, dc, ws, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dh.cpu().numpy(), exp)


def _ragged(oracle, seed, n_batches=5, cap=300):
    return workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=n_batches,
                                 total_packet_cap=cap, seed=seed)


def test_sig_batch_mixed_jobs(lib, oracle):
    rs = _ragged(oracle, 64)
    jobs = [(sp, JOB_VERIFY) for sp in rs.verify] + [(sp, JOB_SIGN) for sp in rs.sign]
    exp = [oracle.verify_packets(sp, nthreads()) for sp in rs.verify] + \
          [oracle.sign_packets(sp, nthreads()) for sp in rs.sign]
    for rep in range(3):                      # graph capture, then replays
        outs = lib.ed25519_batch(jobs)
        for k, (o, e) in enumerate(zip(outs, exp)):
            assert np.array_equal(o, e), (rep, k)
    # interleaved kinds and a different shape
    jobs2 = [jobs[-1], jobs[0], jobs[-2], jobs[1]]
    outs = lib.ed25519_batch(jobs2)
    for o, k in zip(outs, [len(exp) - 1, 0, len(exp) - 2, 1]):
        assert np.array_equal(o, exp[k])


def test_sig_batch_matches_per_call(lib, oracle):
    rs = _ragged(oracle, 65, n_batches=4, cap=200)
    outs = lib.ed25519_batch([(sp, JOB_VERIFY) for sp in rs.verify])
    for o, sp in zip(outs, rs.verify):
        assert np.array_equal(o, lib.verify_many(sp))


def test_sig_batch_out_of_range_items(lib, oracle):
    sp, _ = workloads.verify_uniform(lib.create_keypairs, lib.sign_many, n=64, seed=66)
    bad = type(sp)(sp.batches, sp.message_size, sp.message_lens.copy(), sp.public_key_offsets.copy(),
                   sp.signature_offsets.copy(), sp.message_start_offsets.copy())
    total = sum(len(b) for b in sp.batches)
    bad.signature_offsets[3] = total - 8
    bad.message_lens[5] = 10 ** 9
    good = lib.verify_many(sp)
    # another job follows: an out-of-range offset must not read into it
    outs = lib.ed25519_batch([(bad, JOB_VERIFY), (sp, JOB_VERIFY)])
    exp = good.copy()
    exp[3] = 0
    exp[5] = 0
    assert np.array_equal(outs[0], exp)
    assert np.array_equal(outs[1], good)


def test_sig_batch_device(lib, oracle):
    torch = pytest.importorskip("torch")
    rs = _ragged(oracle, 67, n_batches=1, cap=400)
    sp, ss = rs.verify[0], rs.sign[0]
    # put both into one device buffer: verify packets then sign packets
    pv, ps = sp.concatenated(), ss.concatenated()
    packets = np.concatenate([pv, ps])
    off = np.uint32(len(pv))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    v = [dev(a.astype(np.int32)) for a in (sp.message_lens, sp.public_key_offsets, sp.signature_offsets,
                                           sp.message_start_offsets)]
    s = [dev(a.astype(np.int32)) for a in (ss.message_lens, ss.public_key_offsets + off, ss.signature_offsets + off,
                                           ss.message_start_offsets + off)]
    v_out = torch.zeros(sp.total_signatures, dtype=torch.uint8, device="cuda")
    s_out = torch.zeros((ss.total_signatures, 64), dtype=torch.uint8, device="cuda")
    q = torch.zeros(4, dtype=torch.int32, device="cuda")
    lib.ed25519_batch_device(dev(packets), v, v_out, s, s_out, q, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(v_out.cpu().numpy(), oracle.verify_packets(sp, nthreads()))
    assert np.array_equal(s_out.cpu().numpy(), oracle.sign_packets(ss, nthreads()))


def test_tuning_report(lib):
    t = lib.tuning()
    assert t["sig_threads"] in (64, 128, 256)
    assert t["verify_window"] in (0, 4)                 # half-size scalars or the 4-bit window
    assert set(t["sig_calibration_ms"]) == {"half", "w4"}
    assert t["poh_warps_per_smsp"] in (1, 2)
    assert t["poh_paired"] in (0, 1)
    assert t["sms"] > 0


@pytest.mark.parametrize("form,warps_per_sm", [(0, 4), (0, 8), (0, 1), (1, 4), (2, 4), (2, 8), (2, 2),
                                               (3, 4), (3, 2), (4, 4), (5, 4)])
def test_poh_batch_every_launch_shape(lib, oracle, form, warps_per_sm):
    """Single, packed, paired and packed-paired persistent forms, at several
    residencies (odd pair counts included), give the oracle's chains (ragged
    and zero counts, more chains than resident lanes so lanes refill)."""
    torch = pytest.importorskip("torch")
    h, cnt = workloads.poh_ragged(n=25000, max_hashes=400, seed=68 + form)
    cnt[:5] = [0, 0, 1, 400, 2]
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    sms = lib.tuning()["sms"]
    dh = torch.from_numpy(h.copy()).cuda()
    dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
    ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
    warps = warps_per_sm * sms + (2 if form >= 2 else 0)   # + one pair: odd pair count per block
    lib.poh_verify_batch_shape(dh, dc, ws, warps, form, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dh.cpu().numpy(), exp)


@pytest.mark.parametrize("form", [0, 1, 2, 3, 4, 5])
def test_poh_batch_forms_few_chains(lib, oracle, form):
    """Fewer chains than one warp (a partly empty pair and block)."""
    torch = pytest.importorskip("torch")
    h, cnt = workloads.poh_ragged(n=37, max_hashes=3000, seed=90 + form)
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    dh = torch.from_numpy(h.copy()).cuda()
    dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
    ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
    lib.poh_verify_batch_shape(dh, dc, ws, 608, form, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dh.cpu().numpy(), exp)


def test_poh_batch_shape_rejects_bad_shapes(lib):
    torch = pytest.importorskip("torch")
    dh = torch.zeros((4, 32), dtype=torch.uint8, device="cuda")
    dc = torch.ones(4, dtype=torch.int64, device="cuda")
    ws = torch.empty(lib.poh_batch_workspace_size(4), dtype=torch.uint8, device="cuda")
    for warps, form in ((0, 0), (64, 6), (64, -1), (10 ** 6, 0)):
        with pytest.raises(RuntimeError):
            lib.poh_verify_batch_shape(dh, dc, ws, warps, form)


@pytest.mark.parametrize("uniform", [True, False])
def test_poh_batch_device_chooses_shape(lib, oracle, uniform):
    """The device form picks paired or single warps from the counts on the
    device: uniform counts over many chains (single warps: the total bounds
    the makespan) and ragged ones (paired: the longest chain does); both
    through the shape entry point (form 5) and the tuned device entry."""
    torch = pytest.importorskip("torch")
    sms = lib.tuning()["sms"]
    n = 4 * sms * 32 * 2 + 13
    h, cnt = workloads.poh_ragged(n=n, max_hashes=600, seed=71 + uniform)
    if uniform:
        cnt[:] = 600
    cnt[:3] = [0, 1, 600]
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    for shape in (True, False):
        dh = torch.from_numpy(h.copy()).cuda()
        dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
        ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        if shape:
            lib.poh_verify_batch_shape(dh, dc, ws, 4 * sms, lib.POH_AUTO, st)
        else:
            lib.poh_verify_batch_device(dh, dc, ws, st)
        torch.cuda.synchronize()
        assert np.array_equal(dh.cpu().numpy(), exp), shape


def test_sig_batch_both_verify_modes(lib, oracle):
    """The persistent launch verifies four lanes per signature up to 64 per
    SM and one lane per signature above: a batch on each side of the rule,
    against the oracle."""
    sms = lib.tuning()["sms"]
    for n in (8 * sms, 64 * sms + 100):
        sp, corrupted = workloads.verify_uniform(lib.create_keypairs, lib.sign_many, n=n, seed=70 + n % 7)
        exp = oracle.verify_packets(sp, nthreads())
        got = lib.ed25519_batch([(sp, JOB_VERIFY)])[0]
        assert np.array_equal(got, exp), n
        assert np.array_equal(lib.verify_many(sp), exp), n
        assert np.array_equal(got.astype(bool), ~corrupted)


def test_sig_batch_window4_form(oracle, tmp_path):
    """The 4-bit-window one-lane form in the batched kernel (the autotuner
    normally keeps half-size scalars; GB300_CRYPT_VERIFY_WINDOW=4 forces the
    window, read once per process, so a child process runs it) gives the
    oracle's verdicts."""
    import os
    import subprocess
    import sys
    rs = _ragged(oracle, 71, n_batches=3, cap=300)
    script = f"""
import sys, numpy as np
sys.path[:0] = {[os.path.dirname(os.path.abspath(__file__)), os.path.dirname(os.path.dirname(os.path.abspath(__file__))), os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "solana-perf-libs_gb300")]!r}
import cuda_crypt, workloads
from cuda_crypt import JOB_VERIFY
from oracle.oracle import get_oracle
o = get_oracle()
rs = workloads.ragged_sigs(o.create_keypairs, o.sign_packets, n_batches=3, total_packet_cap=300, seed=71)
lib = cuda_crypt.get_lib()
assert lib.init()
assert lib.tuning()["verify_window"] == 4
outs = lib.ed25519_batch([(sp, JOB_VERIFY) for sp in rs.verify])
np.save({str(tmp_path / "v.npy")!r}, np.concatenate(outs))
"""
    env = dict(os.environ, GB300_CRYPT_VERIFY_WINDOW="4")
    subprocess.run([sys.executable, "-c", script], env=env, check=True, timeout=600)
    got = np.load(tmp_path / "v.npy")
    exp = np.concatenate([oracle.verify_packets(sp, nthreads()) for sp in rs.verify])
    assert np.array_equal(got, exp)


def test_sig_batch_mixed_order_keys(lib, oracle):
    """Keys and nonces with small-order components in the batched kernel:
    four lanes (a launch within the four-lane limit) and one lane with
    half-size scalars (the same items beside enough others to pass it)."""
    from test_gpu_verify import pack_items
    from test_gpu_verify_quad import _valid_items, mixed_order_items
    sms = lib.tuning()["sms"]
    mixed = mixed_order_items(n=96, seed=77)
    filler, _ = _valid_items(oracle, 64 * sms + 200, 78, msg_len=32)
    small = pack_items(mixed, gap_seed=12)
    big = pack_items(mixed + filler, gap_seed=13)
    out = lib.ed25519_batch([(small, JOB_VERIFY)])[0]
    assert np.array_equal(out, oracle.verify_packets(small, nthreads()))
    out = lib.ed25519_batch([(big, JOB_VERIFY)])[0]
    assert np.array_equal(out, oracle.verify_packets(big, nthreads()))
