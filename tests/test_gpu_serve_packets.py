"""Wire-format packet batches in the served loop (gb300_server_submit_packets):
each batch gets exactly the packet verdicts and signature counts of the
one-call gb300_ed25519_verify_packets (and of the oracle), whether it runs
alone, merged with other batches of its stride, beside batches of another
stride, offset-form verify / sign jobs and PoH, from page-locked or pageable
buffers; invalid batches are refused with ticket 0."""
import ctypes
import threading

import numpy as np
import pytest

import workloads
from cuda_crypt import JOB_SIGN, JOB_VERIFY, GpuElems, Server
from conftest import nthreads

pytestmark = pytest.mark.gpu


def _wire(oracle, n, seed, stride=workloads.WIRE_STRIDE, **kw):
    return workloads.wire_packets(oracle.create_keypairs, oracle.sign_packets, n=n, seed=seed, stride=stride, **kw)


@pytest.fixture(scope="module")
def wires(oracle):
    ws = [_wire(oracle, n, 90 + k, corrupt_frac=0.1, malformed_frac=0.05)
          for k, n in enumerate([1, 37, 600, 2100, 5])]
    ws.append(_wire(oracle, 300, 99, stride=1237, corrupt_frac=0.1, malformed_frac=0.05))
    ws.append(_wire(oracle, 64, 100, malformed_frac=1.0))
    return ws


def _expected(oracle, w):
    exp, _, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens, nthreads())
    return exp, counts


def test_packets_alone_match_one_call_and_oracle(lib, oracle, wires):
    srv = Server(lib)
    try:
        for k, w in enumerate(wires):
            exp, counts = _expected(oracle, w)
            one, one_counts = lib.verify_packets(w.data, w.lens)
            assert np.array_equal(one, exp) and np.array_equal(one_counts, counts), k
            t, out, cnt = srv.submit_packets(w.data, w.lens, batches=1 + k % 3)
            assert t and srv.wait(t, 60000) == 1, k
            assert np.array_equal(out, exp) and np.array_equal(cnt, counts), k
    finally:
        srv.close()


def test_packets_in_the_mix(lib, oracle, wires):
    """Packet batches of two strides, offset verify and sign jobs and PoH
    submitted together from three threads."""
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=4, total_packet_cap=200,
                               seed=101)
    ver = [lib.verify_many(sp) for sp in rs.verify]
    sig = [lib.sign_many(sp) for sp in rs.sign]
    h, c = workloads.poh_ragged(n=48, max_hashes=2000, seed=102)
    poh = h.ravel().copy()
    assert lib.poh_verify_many(poh, c) == 0
    pexp = [_expected(oracle, w) for w in wires]
    srv = Server(lib)
    try:
        results, lock = {}, threading.Lock()

        def submit(items):
            for kind, k in items:
                if kind == "w":
                    t, out, cnt = srv.submit_packets(wires[k].data, wires[k].lens, batches=2)
                    res = (out, cnt)
                elif kind == "v":
                    t, res = srv.submit_sigs(rs.verify[k], JOB_VERIFY)
                elif kind == "s":
                    t, res = srv.submit_sigs(rs.sign[k], JOB_SIGN)
                else:
                    res = h.ravel().copy()
                    t = srv.submit_poh(res, c)
                assert t
                with lock:
                    results[(kind, k)] = (t, res)

        work = [("w", k) for k in range(len(wires))] + [("v", k) for k in range(len(rs.verify))] + \
               [("s", k) for k in range(len(rs.sign))] + [("p", 0)]
        ths = [threading.Thread(target=submit, args=(work[i::3],)) for i in range(3)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        for (kind, k), (t, res) in results.items():
            assert srv.wait(t, 60000) == 1, (kind, k)
            if kind == "w":
                assert np.array_equal(res[0], pexp[k][0]) and np.array_equal(res[1], pexp[k][1]), k
            else:
                exp = ver[k] if kind == "v" else sig[k] if kind == "s" else poh
                assert np.array_equal(res, exp), (kind, k)
        kinds = {e[0] for e in srv.trace()}
        # wire packets in slot launches (3), offset-form jobs on the resident
        # signature service (4), PoH (2)
        assert 3 in kinds and 4 in kinds and 2 in kinds
    finally:
        srv.close()


def test_packets_merge_by_stride_and_page_locked(lib, oracle, wires):
    """With one signature slot and a backlog, batches of one stride merge
    into shared launches; page-locked batches are copied directly."""
    same = [w for w in wires if w.stride == workloads.WIRE_STRIDE]
    exp = [_expected(oracle, w) for w in same]
    regs = [w.data for w in same[:2]]
    for a in regs:
        assert lib.host_register(a) == 0
    srv = Server(lib, sig_slots=1)
    try:
        subs = [srv.submit_packets(w.data, w.lens) for w in same * 3]
        for i, (t, out, cnt) in enumerate(subs):
            assert t and srv.wait(t, 60000) == 1, i
            e, ec = exp[i % len(same)]
            assert np.array_equal(out, e) and np.array_equal(cnt, ec), i
        st = srv.stats()
        assert st["max_requests_merged"] > 1 and st["launches_sig"] < len(subs)
        tr = [e for e in srv.trace() if e[0] == 3]
        assert sum(e[1] for e in tr) == len(subs)
        assert sum(e[2] for e in tr) == 3 * sum(len(w.lens) for w in same)
    finally:
        srv.close()
        for a in regs:
            lib.host_unregister(a)


def test_packets_without_counts(lib, oracle, wires):
    w = wires[2]
    exp, _ = _expected(oracle, w)
    srv = Server(lib)
    try:
        t, out, cnt = srv.submit_packets(w.data, w.lens, counts=False)
        assert cnt is None and t and srv.wait(t, 60000) == 1
        assert np.array_equal(out, exp)
    finally:
        srv.close()


def test_packets_refused(lib, wires):
    w = wires[1]
    srv = Server(lib)
    small = Server(lib, device_memory_cap=4096)
    try:
        L = lib.lib
        u8, u32 = ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_uint32)
        lens = np.ascontiguousarray(w.lens, dtype=np.uint32)
        out = np.zeros(len(lens), dtype=np.uint8)
        el = (GpuElems * 1)()
        el[0].elems = None
        el[0].num = 3                                          # a run with packets but no data
        lp, op = lens.ctypes.data_as(u32), out.ctypes.data_as(u8)
        assert L.gb300_server_submit_packets(srv.h, el, 1, w.stride, lp, op, None) == 0
        el[0].num = 0                                          # no packets at all
        assert L.gb300_server_submit_packets(srv.h, el, 1, w.stride, lp, op, None) == 0
        el[0].elems = w.data.ctypes.data_as(u8)
        el[0].num = len(lens)
        assert L.gb300_server_submit_packets(srv.h, el, 1, 0, lp, op, None) == 0          # stride 0
        assert L.gb300_server_submit_packets(srv.h, el, 1, w.stride, None, op, None) == 0  # no lengths
        assert L.gb300_server_submit_packets(srv.h, el, 1, w.stride, lp, None, None) == 0  # no output
        # slot bytes of 4 GiB or more (refused before any data is read)
        assert L.gb300_server_submit_packets(srv.h, el, 1, 1 << 31, lp, op, None) == 0
        t, _, _ = small.submit_packets(w.data, w.lens)        # alone above the memory cap
        assert t == 0
    finally:
        small.close()
        srv.close()
