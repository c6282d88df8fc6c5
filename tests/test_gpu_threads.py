"""The C ABI called from many host threads at once (the reference's calls
are reentrant: a global lock picks a (GPU, queue) context round-robin and a
per-context lock serialises its users, src/cuda-ecc-ed25519/gpu_ctx.cu:
46-73).  Eight threads interleave verify_many, sign_many, poh_verify_many,
the batched entry points and the wire-packet path on different inputs;
every result equals the same call made alone."""
import threading

import numpy as np
import pytest

import workloads
from cuda_crypt import JOB_SIGN, JOB_VERIFY

pytestmark = pytest.mark.gpu


def test_concurrent_calls_match_alone(lib, oracle):
    rs = workloads.ragged_sigs(oracle.create_keypairs, oracle.sign_packets, n_batches=6, total_packet_cap=200,
                               seed=81)
    pohs = [workloads.poh_ragged(n=n, max_hashes=2000, seed=82 + n) for n in (5, 64, 300)]
    wire = workloads.wire_packets(oracle.create_keypairs, oracle.sign_packets, n=300, seed=83)
    exp_v = [lib.verify_many(sp) for sp in rs.verify]
    exp_s = [lib.sign_many(sp) for sp in rs.sign[:6]]
    exp_p = []
    for h, c in pohs:
        b = h.ravel().copy()
        assert lib.poh_verify_many(b, c) == 0
        exp_p.append(b)
    exp_w, exp_wc = lib.verify_packets(wire.data, wire.lens)
    jobs = [(sp, JOB_VERIFY) for sp in rs.verify[:3]] + [(sp, JOB_SIGN) for sp in rs.sign[:3]]
    exp_b = lib.ed25519_batch(jobs)
    errors = []

    def worker(tid):
        try:
            rng = np.random.default_rng(tid)
            for it in range(12):
                op = int(rng.integers(0, 5))
                if op == 0:
                    k = int(rng.integers(0, len(rs.verify)))
                    assert np.array_equal(lib.verify_many(rs.verify[k]), exp_v[k]), ("verify", k)
                elif op == 1:
                    k = int(rng.integers(0, len(exp_s)))
                    assert np.array_equal(lib.sign_many(rs.sign[k]), exp_s[k]), ("sign", k)
                elif op == 2:
                    k = int(rng.integers(0, len(pohs)))
                    h, c = pohs[k]
                    b = h.ravel().copy()
                    assert lib.poh_verify_many(b, c) == 0
                    assert np.array_equal(b, exp_p[k]), ("poh", k)
                elif op == 3:
                    got = lib.ed25519_batch(jobs)
                    assert all(np.array_equal(a, e) for a, e in zip(got, exp_b)), "batch"
                else:
                    out, cnt = lib.verify_packets(wire.data, wire.lens)
                    assert np.array_equal(out, exp_w) and np.array_equal(cnt, exp_wc), "packets"
        except Exception as e:          # collected, reported by the main thread
            errors.append((tid, repr(e)))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(300)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors[:5]
