"""PoH chain verification on the GPU (poh_verify_many and the device form)
against the reference's golden vectors and the CPU oracle.  Bit-exact."""
import numpy as np
import pytest

import workloads
from conftest import nthreads

pytestmark = pytest.mark.gpu


def _golden_arrays(g):
    h = np.array([list(bytes.fromhex(x)) for x in g["hashes"]], dtype=np.uint8)
    e = np.array([list(bytes.fromhex(x)) for x in g["expected"]], dtype=np.uint8)
    return h, np.array(g["num_hashes"], dtype=np.uint64), e


def test_poh_golden_332(lib, golden_poh):
    h, n, e = _golden_arrays(golden_poh)
    buf = h.ravel().copy()
    assert lib.poh_verify_many(buf, n) == 0
    assert np.array_equal(buf.reshape(-1, 32), e)


@pytest.mark.parametrize("stream", [0, 1])
def test_poh_random_counts(lib, oracle, stream):
    rng = np.random.default_rng(11)
    n = 777                                        # not a multiple of the block size
    h = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    cnt = rng.integers(0, 3000, n).astype(np.uint64)
    cnt[:5] = [0, 1, 2, 63, 64]
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    buf = h.ravel().copy()
    assert lib.poh_verify_many(buf, cnt, use_non_default_stream=stream) == 0
    assert np.array_equal(buf.reshape(-1, 32), exp)


def test_poh_empty_and_zero(lib):
    buf = np.zeros(32, dtype=np.uint8)
    assert lib.poh_verify_many(buf[:0], np.zeros(0, dtype=np.uint64)) == 0
    rng = np.random.default_rng(12)
    h = rng.integers(0, 256, 64, dtype=np.uint8)
    keep = h.copy()
    assert lib.poh_verify_many(h, np.zeros(2, dtype=np.uint64)) == 0
    assert np.array_equal(h, keep)


def test_poh_uniform_full_size(lib, oracle):
    """4096 entries x 12500 hashes, with 5% of the expected hashes corrupted:
    final hashes bit-exact and pass/fail flags exactly the uncorrupted set."""
    h, cnt = workloads.poh_uniform()
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    exp_bad, mask = workloads.corrupt_expected(exp, 0.05, seed=21)
    buf = h.ravel().copy()
    assert lib.poh_verify_many(buf, cnt) == 0
    got = buf.reshape(-1, 32)
    assert np.array_equal(got, exp)
    flags = np.all(got == exp_bad, axis=1)
    assert np.array_equal(flags, ~mask)


def test_poh_device_form(lib, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(13)
    n = 300
    h = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    cnt = rng.integers(0, 500, n).astype(np.uint64)
    exp = oracle.poh_verify_many(h, cnt, nthreads())
    dh = torch.from_numpy(h.copy()).cuda()
    dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
    lib.poh_verify_device(dh, dc, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dh.cpu().numpy(), exp)
