"""gb300_poh_verify_batch_static: the ragged-batch PoH entry point for callers
that cannot allocate GPU memory (its scratch is a device array built into the
library).  Checked through the C ABI against the existing workspace-taking
entry point, on two calls in a row.  Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu


def _static(lib):
    f = lib.lib.gb300_poh_verify_batch_static
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_static_scratch_matches_workspace_entry_point(lib):
    torch = pytest.importorskip("torch")
    static = _static(lib)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):                               # two calls in a row share the array
        h, cnt = workloads.poh_ragged(n=3000 + 1000 * call, max_hashes=4000, seed=80 + call)
        cnt[:3] = [0, 1, 4000]
        dc = torch.from_numpy(cnt.astype(np.int64)).cuda()
        a = torch.from_numpy(h.copy()).cuda()
        b = torch.from_numpy(h.copy()).cuda()
        ws = torch.empty(lib.poh_batch_workspace_size(len(cnt)), dtype=torch.uint8, device="cuda")
        lib.poh_verify_batch_device(a, dc, ws, stream)
        assert static(b.data_ptr(), dc.data_ptr(), len(cnt), stream) == 0
        torch.cuda.synchronize()
        assert np.array_equal(a.cpu().numpy(), b.cpu().numpy()), call
        assert not np.array_equal(b.cpu().numpy()[2], h[2])       # the chains did run


def test_static_scratch_rejects_oversize(lib):
    torch = pytest.importorskip("torch")
    static = _static(lib)
    n = 262144 + 1
    h = torch.zeros((n, 32), dtype=torch.uint8, device="cuda")
    c = torch.ones(n, dtype=torch.int64, device="cuda")
    assert static(h.data_ptr(), c.data_ptr(), n, torch.cuda.current_stream().cuda_stream) != 0
    torch.cuda.synchronize()
    assert int(h.abs().sum().item()) == 0                      # nothing ran
