"""gb300_poh_verify_batch_static: the ragged-batch PoH entry point for callers
that cannot allocate GPU memory (its scratch is a device array built into the
library).  Checked through the C ABI against the CPU oracle and against the
workspace-taking entry point, on calls in a row that share the array: a
ragged batch, a batch whose counts make the device choose single warps
instead of pairs, and a batch of exactly the 262,144-entry limit.  Kept in
its own file, collected last."""
import ctypes

import numpy as np
import pytest

import workloads
from conftest import nthreads

pytestmark = pytest.mark.gpu

STATIC_MAX_ENTRIES = 262144


def _static(lib):
    f = lib.lib.gb300_poh_verify_batch_static
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _run_both(lib, static, torch, h, cnt):
    """(static entry point's final hashes, workspace entry point's)."""
    stream = torch.cuda.current_stream().cuda_stream
    dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
    a = torch.from_numpy(h.copy()).cuda()
    b = torch.from_numpy(h.copy()).cuda()
    ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
    lib.poh_verify_batch_device(a, dc, ws, stream)
    assert static(b.data_ptr(), dc.data_ptr(), len(cnt), stream) == 0
    torch.cuda.synchronize()
    return b.cpu().numpy(), a.cpu().numpy()


def test_static_scratch_matches_oracle_and_workspace_entry_point(lib, oracle):
    torch = pytest.importorskip("torch")
    static = _static(lib)
    for call in range(2):                               # two calls in a row share the array
        h, cnt = workloads.poh_ragged(n=3000 + 1000 * call, max_hashes=4000, seed=80 + call)
        cnt[:3] = [0, 1, 4000]
        got, ws_out = _run_both(lib, static, torch, h, cnt)
        assert np.array_equal(got, oracle.poh_verify_many(h, cnt, nthreads())), call
        assert np.array_equal(got, ws_out), call
        assert np.array_equal(got[0], h[0])             # count 0: unchanged
        assert not np.array_equal(got[2], h[2])         # the chains did run


def test_static_scratch_single_warp_shape(lib, oracle):
    """200,000 entries of 40..60 hashes: bound by the total work, so the
    device's shape rule picks single warps (estimate ~1.3 M cycles against
    ~2.0 M for pairs at 152 SMs) and re-arms the queue for them.  The call
    before it left a paired-shape header in the shared array."""
    torch = pytest.importorskip("torch")
    static = _static(lib)
    rng = np.random.default_rng(83)
    h0, c0 = workloads.poh_ragged(n=2000, max_hashes=3000, seed=82)
    got0, _ = _run_both(lib, static, torch, h0, c0)
    assert np.array_equal(got0, oracle.poh_verify_many(h0, c0, nthreads()))
    n = 200_000
    h = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    cnt = rng.integers(40, 61, n).astype(np.uint64)
    cnt[7] = 0
    got, ws_out = _run_both(lib, static, torch, h, cnt)
    assert np.array_equal(got, oracle.poh_verify_many(h, cnt, nthreads()))
    assert np.array_equal(got, ws_out)
    assert np.array_equal(got[7], h[7])


def test_static_scratch_at_the_entry_limit(lib, oracle):
    torch = pytest.importorskip("torch")
    static = _static(lib)
    rng = np.random.default_rng(84)
    n = STATIC_MAX_ENTRIES
    h = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    cnt = rng.integers(0, 17, n).astype(np.uint64)
    cnt[-1] = 300                                       # the last entry is the longest
    got, ws_out = _run_both(lib, static, torch, h, cnt)
    assert np.array_equal(got, oracle.poh_verify_many(h, cnt, nthreads()))
    assert np.array_equal(got, ws_out)


def test_static_scratch_rejects_oversize(lib):
    torch = pytest.importorskip("torch")
    static = _static(lib)
    n = STATIC_MAX_ENTRIES + 1
    h = torch.zeros((n, 32), dtype=torch.uint8, device="cuda")
    c = torch.ones(n, dtype=torch.int64, device="cuda")
    assert static(h.data_ptr(), c.data_ptr(), n, torch.cuda.current_stream().cuda_stream) != 0
    torch.cuda.synchronize()
    assert int(h.abs().sum().item()) == 0                      # nothing ran
