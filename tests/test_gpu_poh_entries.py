"""Solana ledger entries on the GPU (include/poh_verify.h): recording chains
of entries and verifying entries with transaction mixins, host and device
forms, against the CPU oracle's restatement of the entry rule (itself
checked against hashlib in tests/test_oracle.py)."""
import numpy as np
import pytest

import workloads
from conftest import nthreads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ledger(oracle):
    w = workloads.poh_entries(chains=96, entries_per_chain=40, tick_hashes=2000, seed=41)
    w.expected, last = oracle.poh_record(w.start, w.first, w.num_hashes, w.mixins, w.has_mixin)
    return w, last


def test_record_host(lib, ledger):
    w, last = ledger
    rec, got_last = lib.poh_record(w.start, w.first, w.num_hashes, w.mixins, w.has_mixin)
    assert np.array_equal(rec, w.expected) and np.array_equal(got_last, last)


def test_record_device_ragged_chains(lib, oracle):
    """Chains of different lengths, an empty chain and a chain of one entry."""
    torch = pytest.importorskip("torch")
    w = workloads.poh_entries(chains=6, entries_per_chain=10, tick_hashes=500, seed=42)
    first = np.array([0, 10, 10, 11, 30, 45, 60], dtype=np.uint64)       # 6 chains: 10, 0, 1, 19, 15, 15
    exp, last = oracle.poh_record(w.start, first, w.num_hashes, w.mixins, w.has_mixin)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    h = dev(w.start.copy())
    out = torch.zeros((len(w.num_hashes), 32), dtype=torch.uint8, device="cuda")
    lib.poh_record_device(h, dev(first.astype(np.int64)), dev(w.num_hashes.astype(np.int64)), dev(w.mixins),
                          dev(w.has_mixin), out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), exp)
    assert np.array_equal(h.cpu().numpy(), last)
    assert np.array_equal(last[1], w.start[1])                         # the empty chain keeps its hash


def test_verify_entries_host(lib, oracle, ledger):
    """3% of the recorded hashes and 2% of the mixins corrupted: exactly
    those entries fail."""
    w, _ = ledger
    rng = np.random.default_rng(43)
    exp = w.expected.copy()
    mix = w.mixins.copy()
    bad_hash = rng.random(len(exp)) < 0.03
    bad_mix = (rng.random(len(exp)) < 0.02) & (w.has_mixin == 1)
    exp[bad_hash, 5] ^= 0x10
    mix[bad_mix, 30] ^= 0x01
    start = w.entry_start()
    ok = lib.poh_verify_entries(start, w.num_hashes, mix, w.has_mixin, exp)
    ok_o, _ = oracle.poh_verify_entries(start, w.num_hashes, mix, w.has_mixin, exp, nthreads())
    assert np.array_equal(ok, ok_o)
    assert np.array_equal(ok.astype(bool), ~(bad_hash | bad_mix))


def test_verify_entries_device(lib, oracle, ledger):
    torch = pytest.importorskip("torch")
    w, _ = ledger
    start = w.entry_start()
    exp = w.expected.copy()
    exp[::97, 0] ^= 0xff
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    n = len(w.num_hashes)
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    out = torch.zeros((n, 32), dtype=torch.uint8, device="cuda")
    ws = torch.empty(lib.poh_entries_workspace_size(n), dtype=torch.uint8, device="cuda")
    lib.poh_verify_entries_device(dev(start), dev(w.num_hashes.astype(np.int64)), dev(w.mixins), dev(w.has_mixin),
                                  dev(exp), ok, out, ws, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ok_o, out_o = oracle.poh_verify_entries(start, w.num_hashes, w.mixins, w.has_mixin, exp, nthreads())
    assert np.array_equal(ok.cpu().numpy(), ok_o) and np.array_equal(out.cpu().numpy(), out_o)
    assert int(ok_o.sum()) == n - len(range(0, n, 97))


def test_verify_entries_edges(lib, oracle):
    """Zero hashes with and without a mixin, one entry, long ticks beside
    short entries (the ragged batch orders them longest first)."""
    rng = np.random.default_rng(44)
    n = 7
    start = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    nh = np.array([0, 0, 1, 1, 20000, 3, 5000], dtype=np.uint64)
    hm = np.array([0, 1, 0, 1, 0, 1, 1], dtype=np.uint8)
    mx = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    _, out = oracle.poh_verify_entries(start, nh, mx, hm, start, 1)
    ok = lib.poh_verify_entries(start, nh, mx, hm, out)
    assert ok.all()
    assert np.array_equal(out[0], start[0])                            # an empty tick changes nothing
    assert lib.poh_verify_entries(start[:1], nh[:1], mx[:1], hm[:1], out[:1]).all()
