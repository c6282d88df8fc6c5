"""The served request loop, with verify/sign jobs on the resident signature
service (the default) and on merged slot launches: requests submitted
together (from several threads, mixed verify / sign / PoH) each get exactly
the result they get alone through the one-call entry points; memory-capped
admission still completes everything; requests above the memory budget are
refused, requests above the per-launch item cap run alone.  Service only:
the kernel is launched again after it leaves when idle, four-lane and
one-lane chunks run side by side, and jobs too large for its rings take the
slot path."""
import os
import threading
import time

import numpy as np
import pytest

import workloads
from cuda_crypt import JOB_SIGN, JOB_VERIFY, SIG_SERVICE, SIG_SLOTS, Server
from conftest import nthreads

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[SIG_SERVICE, SIG_SLOTS], ids=["service", "slots"])
def mode(request):
    return request.param


@pytest.fixture(scope="module")
def mix(lib, oracle):
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=6, total_packet_cap=300, seed=71)
    pohs = [workloads.poh_ragged(n=int(n), max_hashes=3000, seed=72 + k) for k, n in enumerate([40, 7, 200, 64])]
    return rs, pohs


def _alone(lib, rs, pohs):
    ver = [lib.verify_many(sp) for sp in rs.verify]
    sig = [lib.sign_many(sp) for sp in rs.sign]
    poh = []
    for h, c in pohs:
        b = h.ravel().copy()
        assert lib.poh_verify_many(b, c) == 0
        poh.append(b)
    return ver, sig, poh


def test_same_alone_and_in_the_mix(lib, oracle, mix, mode):
    rs, pohs = mix
    ver, sig, poh = _alone(lib, rs, pohs)
    assert np.array_equal(np.concatenate(ver), np.concatenate([oracle.verify_packets(sp, nthreads()) for sp in rs.verify]))
    srv = Server(lib, sig_mode=mode)
    try:
        results = {}
        lock = threading.Lock()

        def submit_range(kinds):
            for kind, k in kinds:
                if kind == "v":
                    t, out = srv.submit_sigs(rs.verify[k], JOB_VERIFY)
                elif kind == "s":
                    t, out = srv.submit_sigs(rs.sign[k], JOB_SIGN)
                else:
                    h, c = pohs[k]
                    out = h.ravel().copy()
                    t = srv.submit_poh(out, c)
                assert t
                with lock:
                    results[(kind, k)] = (t, out)

        work = [("v", k) for k in range(len(rs.verify))] + [("s", k) for k in range(len(rs.sign))] + \
               [("p", k) for k in range(len(pohs))]
        threads = [threading.Thread(target=submit_range, args=(work[i::3],)) for i in range(3)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        for (kind, k), (t, out) in results.items():
            assert srv.wait(t, 60000) == 1, (kind, k)
            exp = ver[k] if kind == "v" else sig[k] if kind == "s" else poh[k]
            assert np.array_equal(out, exp), (kind, k)
        st = srv.stats()
        assert st["requests_done"] == len(work)
    finally:
        srv.close()


def test_memory_cap_admission_and_refusal(lib, mix, mode):
    rs, pohs = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    biggest = max(sum(len(b) for b in sp.batches) for sp in rs.verify)
    srv = Server(lib, device_memory_cap=biggest + (1 << 20), sig_slots=3, sig_mode=mode)
    try:
        tickets = [srv.submit_sigs(sp, JOB_VERIFY) for sp in rs.verify]
        for (t, out), exp in zip(tickets, ver):
            assert t and srv.wait(t, 60000) == 1
            assert np.array_equal(out, exp)
        small = Server(lib, device_memory_cap=4096, sig_mode=mode)
        try:
            t, _ = small.submit_sigs(rs.verify[0], JOB_VERIFY)
            assert t == 0                                  # larger than the whole budget: refused
        finally:
            small.close()
    finally:
        srv.close()


def test_merging_under_backlog(lib, mix, mode):
    """Slots: a backlog merges into few launches.  Service: the backlog is
    in flight at once, in one or few launches of the resident kernel."""
    rs, _ = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    srv = Server(lib, sig_slots=1, sig_mode=mode)
    try:
        sub = [srv.submit_sigs(sp, JOB_VERIFY) for sp in rs.verify * 4]
        for k, (t, out) in enumerate(sub):
            assert srv.wait(t, 60000) == 1
            assert np.array_equal(out, ver[k % len(ver)])
        st = srv.stats()
        assert st["max_requests_merged"] > 1 and st["launches_sig"] < len(sub)
        if mode == SIG_SERVICE:
            assert st["service"]["served"] == len(sub) and st["service"]["max_in_flight"] > 1
    finally:
        srv.close()


def test_request_above_item_cap_runs_alone(lib, mix, mode):
    """A request with more signatures than max_items_per_launch is not
    refused: it runs in a launch of its own, beside merged small ones."""
    rs, _ = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    big = max(range(len(rs.verify)), key=lambda k: rs.verify[k].total_signatures)
    cap = max(1, rs.verify[big].total_signatures // 3)
    srv = Server(lib, max_items_per_launch=cap, sig_slots=2, sig_mode=mode)
    try:
        sub = [(k,) + tuple(srv.submit_sigs(sp, JOB_VERIFY)) for k, sp in enumerate(rs.verify * 2)]
        for k, t, out in sub:
            assert t and srv.wait(t, 60000) == 1
            assert np.array_equal(out, ver[k % len(rs.verify)])
    finally:
        srv.close()


def test_trace_records_gpu_phases(lib, mix, mode):
    """Every completed launch appears in the trace with its host times and
    the GPU time of its copies and kernels; every job the service ran, with
    its submission, publication and completion times and GPU phases."""
    rs, pohs = mix
    srv = Server(lib, sig_mode=mode)
    try:
        subs = [srv.submit_sigs(sp, JOB_VERIFY)[0] for sp in rs.verify]
        h, c = pohs[0]
        subs.append(srv.submit_poh(h.ravel().copy(), c))
        for t in subs:
            assert srv.wait(t, 60000) == 1
        tr = srv.trace()
        assert len(tr) >= 2 and {e[0] for e in tr} == ({4, 2} if mode == SIG_SERVICE else {0, 2})
        for kind, reqs, items, t_admit, t_enq, t_done, ms_in, ms_run, ms_out in tr:
            assert reqs >= 1 and items >= 1 and t_admit <= t_enq <= t_done
            if kind == 4:
                # GPU wait and run times (clocks related at creation, so a
                # wait can read a little below zero), host total
                assert reqs == 1 and ms_in > -1 and ms_run > 0 and ms_out > 0
            else:
                assert ms_in >= 0 and ms_run > 0 and ms_out >= 0
        assert sum(e[1] for e in tr) == len(subs)
    finally:
        srv.close()


class _env:
    """Environment variables set while a server is created."""

    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update({k: str(v) for k, v in self.kv.items()})

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def test_service_relaunch_after_idle(lib, mix):
    """With a 1 ms idle limit the kernel leaves between rounds of requests;
    every round launches it again and completes."""
    rs, _ = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    with _env(GB300_CRYPT_SERVER_IDLE_US=1000):
        srv = Server(lib)
    try:
        for rnd in range(3):
            sub = [srv.submit_sigs(sp, JOB_VERIFY) for sp in rs.verify]
            for k, (t, out) in enumerate(sub):
                assert srv.wait(t, 60000) == 1
                assert np.array_equal(out, ver[k]), (rnd, k)
            time.sleep(0.05)
        st = srv.stats()["service"]
        assert st["launches"] >= 3 and st["served"] == 3 * len(rs.verify)
    finally:
        srv.close()


def test_service_four_lane_and_one_lane_chunks(lib, oracle):
    """A verify job above the four-lane limit (64 per SM) runs one lane per
    signature while small jobs submitted beside it from other threads run
    four lanes each, plus signing jobs; every result equals the oracle's."""
    sms = lib.tuning()["sms"]
    big, _ = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=64 * sms + 500, seed=73)
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=8, total_packet_cap=60, seed=74)
    exp_big = oracle.verify_packets(big, nthreads())
    exp_v = [oracle.verify_packets(sp, nthreads()) for sp in rs.verify]
    exp_s = [oracle.sign_packets(sp, nthreads()) for sp in rs.sign]
    srv = Server(lib)
    try:
        results, lock = [], threading.Lock()

        def small(kind):
            group = rs.verify if kind == JOB_VERIFY else rs.sign
            for k, sp in enumerate(group * 3):
                t, out = srv.submit_sigs(sp, kind)
                with lock:
                    results.append((kind, k % len(group), t, out))

        ths = [threading.Thread(target=small, args=(JOB_VERIFY,)), threading.Thread(target=small, args=(JOB_SIGN,))]
        for th in ths:
            th.start()
        tb, ob = srv.submit_sigs(big, JOB_VERIFY)
        for th in ths:
            th.join()
        assert srv.wait(tb, 60000) == 1 and np.array_equal(ob, exp_big)
        for kind, k, t, out in results:
            assert t and srv.wait(t, 60000) == 1
            assert np.array_equal(out, exp_v[k] if kind == JOB_VERIFY else exp_s[k]), (kind, k)
        assert srv.stats()["service"]["served"] == len(results) + 1
    finally:
        srv.close()


def test_service_job_too_large_for_its_rings_takes_a_slot(lib, oracle):
    """With 1 MiB of page-locked staging, a job of more than 1 MiB of
    pageable packets cannot be staged by the service and runs on the slot
    path; smaller jobs beside it stay on the service."""
    sp, _ = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=8000, msg_len=200, seed=75)
    assert len(sp.concatenated()) > (1 << 20)
    small, _ = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=100, seed=76)
    exp, exp_small = oracle.verify_packets(sp, nthreads()), oracle.verify_packets(small, nthreads())
    with _env(GB300_CRYPT_SERVER_SVC_STAGE_MB=1):
        srv = Server(lib)
    try:
        t1, o1 = srv.submit_sigs(small, JOB_VERIFY)
        t2, o2 = srv.submit_sigs(sp, JOB_VERIFY)
        t3, o3 = srv.submit_sigs(small, JOB_VERIFY)
        for t in (t1, t2, t3):
            assert t and srv.wait(t, 60000) == 1
        assert np.array_equal(o2, exp) and np.array_equal(o1, exp_small) and np.array_equal(o3, exp_small)
        st = srv.stats()
        assert st["service"]["to_slots"] == 1 and st["service"]["served"] == 2
    finally:
        srv.close()


def test_service_mixed_order_keys(lib, oracle):
    """Keys and nonces with small-order components through the service, in
    four-lane chunks (a small job) and in one-lane chunks with half-size
    scalars (the same items at the front of a job above the four-lane
    limit): the oracle's verdicts."""
    from test_gpu_verify import pack_items
    from test_gpu_verify_quad import _valid_items, mixed_order_items
    sms = lib.tuning()["sms"]
    mixed = mixed_order_items(n=96, seed=75)
    filler, _ = _valid_items(oracle, 64 * sms + 200, 76, msg_len=32)
    small = pack_items(mixed, gap_seed=10)
    big = pack_items(mixed + filler, gap_seed=11)
    exp_small = oracle.verify_packets(small, nthreads())
    exp_big = oracle.verify_packets(big, nthreads())
    assert 0 < int(exp_small.sum()) < len(mixed)
    srv = Server(lib)
    try:
        for sp, exp in ((small, exp_small), (big, exp_big)):
            t, out = srv.submit_sigs(sp, JOB_VERIFY)
            assert srv.wait(t, 60000) == 1 and np.array_equal(out, exp)
    finally:
        srv.close()


def test_service_poh_gives_way_to_a_signature_backlog(lib, oracle):
    """PoH launches of the served loop sleep while signature chunks wait
    unclaimed (threshold 1 chunk here): a PoH batch on every pair, then
    three verify jobs of 20,000 signatures that queue more chunks than the
    service has warps.  Every signature verdict is the oracle's and every
    final PoH hash the plain call's (and the oracle's, on a sample)."""
    sp, _ = workloads.verify_uniform(oracle.create_keypairs, oracle.sign_packets, n=20000, msg_len=64, seed=77)
    exp = oracle.verify_packets(sp, nthreads())
    ph, pc = workloads.poh_uniform(4864, 20000, seed=78)
    plain = ph.ravel().copy()
    assert lib.poh_verify_many(plain, pc) == 0
    sample = np.arange(0, 4864, 76)
    assert np.array_equal(plain.reshape(-1, 32)[sample], oracle.poh_verify_many(ph[sample], pc[sample], nthreads()))
    with _env(GB300_CRYPT_SERVER_POH_YIELD=1):
        srv = Server(lib)
    try:
        for rnd in range(2):
            out = ph.ravel().copy()
            tp = srv.submit_poh(out, pc)
            time.sleep(0.005)
            sub = [srv.submit_sigs(sp, JOB_VERIFY) for _ in range(3)]
            for t, o in sub:
                assert t and srv.wait(t, 60000) == 1 and np.array_equal(o, exp), rnd
            assert tp and srv.wait(tp, 60000) == 1
            assert np.array_equal(out, plain), rnd
    finally:
        srv.close()
