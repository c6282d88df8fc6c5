"""The served request loop: requests submitted together (from several
threads, mixed verify / sign / PoH) each get exactly the result they get
alone through the one-call entry points; memory-capped admission still
completes everything; requests above the memory budget are refused, requests
above the per-launch item cap run alone."""
import threading

import numpy as np
import pytest

import workloads
from cuda_crypt import JOB_SIGN, JOB_VERIFY, Server
from conftest import nthreads

pytestmark = pytest.mark.gpu


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


def test_same_alone_and_in_the_mix(lib, oracle, mix):
    rs, pohs = mix
    ver, sig, poh = _alone(lib, rs, pohs)
    assert np.array_equal(np.concatenate(ver), np.concatenate([oracle.verify_packets(sp, nthreads()) for sp in rs.verify]))
    srv = Server(lib)
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


def test_memory_cap_admission_and_refusal(lib, mix):
    rs, pohs = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    biggest = max(sum(len(b) for b in sp.batches) for sp in rs.verify)
    srv = Server(lib, device_memory_cap=biggest + (1 << 20), sig_slots=3)
    try:
        tickets = [srv.submit_sigs(sp, JOB_VERIFY) for sp in rs.verify]
        for (t, out), exp in zip(tickets, ver):
            assert t and srv.wait(t, 60000) == 1
            assert np.array_equal(out, exp)
        small = Server(lib, device_memory_cap=4096)
        try:
            t, _ = small.submit_sigs(rs.verify[0], JOB_VERIFY)
            assert t == 0                                  # larger than the whole budget: refused
        finally:
            small.close()
    finally:
        srv.close()


def test_merging_under_backlog(lib, mix):
    rs, _ = mix
    srv = Server(lib, sig_slots=1)
    try:
        sub = [srv.submit_sigs(sp, JOB_VERIFY) for sp in rs.verify * 4]
        for t, _ in sub:
            assert srv.wait(t, 60000) == 1
        st = srv.stats()
        assert st["max_requests_merged"] > 1 and st["launches_sig"] < len(sub)
    finally:
        srv.close()


def test_request_above_item_cap_runs_alone(lib, mix):
    """A request with more signatures than max_items_per_launch is not
    refused: it runs in a launch of its own, beside merged small ones."""
    rs, _ = mix
    ver = [lib.verify_many(sp) for sp in rs.verify]
    big = max(range(len(rs.verify)), key=lambda k: rs.verify[k].total_signatures)
    cap = max(1, rs.verify[big].total_signatures // 3)
    srv = Server(lib, max_items_per_launch=cap, sig_slots=2)
    try:
        sub = [(k,) + tuple(srv.submit_sigs(sp, JOB_VERIFY)) for k, sp in enumerate(rs.verify * 2)]
        for k, t, out in sub:
            assert t and srv.wait(t, 60000) == 1
            assert np.array_equal(out, ver[k % len(rs.verify)])
    finally:
        srv.close()


def test_trace_records_gpu_phases(lib, mix):
    """Every completed launch appears in the trace with its host times and
    the GPU time of its copies and kernels."""
    rs, pohs = mix
    srv = Server(lib)
    try:
        subs = [srv.submit_sigs(sp, JOB_VERIFY)[0] for sp in rs.verify]
        h, c = pohs[0]
        subs.append(srv.submit_poh(h.ravel().copy(), c))
        for t in subs:
            assert srv.wait(t, 60000) == 1
        tr = srv.trace()
        assert len(tr) >= 2 and {e[0] for e in tr} == {0, 2}
        for kind, reqs, items, t_admit, t_enq, t_done, ms_in, ms_run, ms_out in tr:
            assert reqs >= 1 and items >= 1 and t_admit <= t_enq <= t_done
            assert ms_in >= 0 and ms_run > 0 and ms_out >= 0
        assert sum(e[1] for e in tr) == len(subs)
    finally:
        srv.close()
