"""Solana wire-format packets parsed and verified on the GPU
(gb300_packets.h) against the CPU oracle's parse and verify: packet
verdicts, signatures per packet, the extracted per-signature offset arrays,
several gpu_Elems runs, graph replays, odd strides and malformed packets;
and the packet verdicts against ed25519_verify_many run on the oracle's
offsets."""
import numpy as np
import pytest

import workloads
from cuda_crypt import SigPackets
from conftest import nthreads

pytestmark = pytest.mark.gpu


def _wire(oracle, n, seed, stride=workloads.WIRE_STRIDE, **kw):
    return workloads.wire_packets(oracle.create_keypairs, oracle.sign_packets, n=n, seed=seed, stride=stride, **kw)


def test_verify_packets_host(lib, oracle):
    w = _wire(oracle, 3000, 31, corrupt_frac=0.08, malformed_frac=0.06)
    exp, _, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens, nthreads())
    for rep in range(3):                       # capture, then graph replays
        out, got_counts = lib.verify_packets(w.data, w.lens, batches=1 + rep)
        assert np.array_equal(out, exp), rep
        assert np.array_equal(got_counts, counts), rep
    assert exp.sum() > 0.8 * len(exp) and (counts == 0).sum() > 0


def test_verify_packets_matches_verify_many(lib, oracle):
    w = _wire(oracle, 700, 32, corrupt_frac=0.2, malformed_frac=0.05)
    counts, ml, ko, so, mo = oracle.wire_offsets(w.data, w.stride, w.lens)
    sp = SigPackets([w.data.ravel().copy()], w.stride, ml, ko, so, mo)
    per_sig = lib.verify_many(sp)
    pkt = np.repeat(np.arange(len(counts)), counts)
    bad = np.zeros(len(counts), dtype=np.int64)
    np.add.at(bad, pkt, (per_sig == 0).astype(np.int64))
    exp = ((counts > 0) & (bad == 0)).astype(np.uint8)
    out, _ = lib.verify_packets(w.data, w.lens)
    assert np.array_equal(out, exp)


@pytest.mark.parametrize("stride", [1232, 1237, 2048])
def test_verify_packets_strides(lib, oracle, stride):
    w = _wire(oracle, 257, 33 + stride, stride=stride)
    exp, _, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens, nthreads())
    out, got = lib.verify_packets(w.data, w.lens)
    assert np.array_equal(out, exp) and np.array_equal(got, counts)


def test_extract_offsets_device(lib, oracle):
    torch = pytest.importorskip("torch")
    w = _wire(oracle, 2500, 34, malformed_frac=0.05)
    counts, ml, ko, so, mo = oracle.wire_offsets(w.data, w.stride, w.lens)
    n, stride = w.data.shape
    cap = lib.packets_signature_capacity(n, stride)
    assert cap >= counts.sum()
    d = torch.from_numpy(w.data.ravel().copy()).cuda()
    dl = torch.from_numpy(w.lens.astype(np.int32)).cuda()
    ws = torch.empty(lib.packets_workspace_size(n, stride), dtype=torch.uint8, device="cuda")
    arrs = [torch.full((cap,), 0x7fffffff, dtype=torch.int32, device="cuda") for _ in range(4)]
    dc = torch.zeros(n, dtype=torch.int32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.extract_offsets_device(d, stride, dl, ws, *arrs, counts=dc, total=tot,
                               stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    t = int(tot.item())
    assert t == counts.sum()
    assert np.array_equal(dc.cpu().numpy().astype(np.uint32), counts)
    for a, e in zip(arrs, (ml, ko, so, mo)):
        assert np.array_equal(a[:t].cpu().numpy().astype(np.uint32), e)


def test_verify_packets_device(lib, oracle):
    torch = pytest.importorskip("torch")
    w = _wire(oracle, 1500, 35, corrupt_frac=0.1, malformed_frac=0.1)
    exp, _, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens, nthreads())
    n, stride = w.data.shape
    d = torch.from_numpy(w.data.ravel().copy()).cuda()
    dl = torch.from_numpy(w.lens.astype(np.int32)).cuda()
    ws = torch.empty(lib.packets_workspace_size(n, stride), dtype=torch.uint8, device="cuda")
    out = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    dc = torch.zeros(n, dtype=torch.int32, device="cuda")
    lib.verify_packets_device(d, stride, dl, ws, out, dc, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), exp)
    assert np.array_equal(dc.cpu().numpy().astype(np.uint32), counts)


def test_verify_packets_edges(lib, oracle):
    # all malformed; a single packet; zero packets; more than one scan block
    w = _wire(oracle, 40, 36, malformed_frac=1.0)
    out, counts = lib.verify_packets(w.data, w.lens)
    assert not out.any() and not counts.any()
    w1 = _wire(oracle, 1, 37, malformed_frac=0.0, corrupt_frac=0.0)
    assert lib.verify_packets(w1.data, w1.lens)[0][0] == 1
    empty = np.zeros((0, 1280), dtype=np.uint8)
    out, counts = lib.verify_packets(empty, np.zeros(0, dtype=np.uint32))
    assert out.size == 0
    big = _wire(oracle, 5000, 38, malformed_frac=0.02)
    exp, _, counts = oracle.verify_wire_packets(big.data, big.stride, big.lens, nthreads())
    out, got = lib.verify_packets(big.data, big.lens, batches=4)
    assert np.array_equal(out, exp) and np.array_equal(got, counts)


@pytest.mark.parametrize("n", [2000, 2800])
def test_verify_packets_form_by_device_count(lib, oracle, n):
    """Four signers per packet: 8,000 and 11,200 signatures in launches sized
    by capacity (20 per packet) for either verify form, so the kernel picks
    the form from the parsed count (four lanes up to 64 per SM, else one)."""
    w = _wire(oracle, n, 39 + n, corrupt_frac=0.05, malformed_frac=0.02, signers=(4,))
    exp, _, counts = oracle.verify_wire_packets(w.data, w.stride, w.lens, nthreads())
    assert counts.max() == 4
    out, got = lib.verify_packets(w.data, w.lens)
    assert np.array_equal(out, exp) and np.array_equal(got, counts)


def _fuzzed(oracle, n, seed):
    return workloads.fuzz_wire(_wire(oracle, n, seed, corrupt_frac=0.0, malformed_frac=0.0), seed)


@pytest.mark.parametrize("seed", [201, 202])
def test_extract_offsets_fuzzed(lib, oracle, seed):
    """The device parse against the oracle's on fuzzed packets: per-packet
    signature counts and the four per-signature arrays."""
    torch = pytest.importorskip("torch")
    data, lens = _fuzzed(oracle, 3000, seed)
    counts, ml, ko, so, mo = oracle.wire_offsets(data, data.shape[1], lens)
    assert (counts == 0).sum() > 300 and (counts > 0).sum() > 1000
    n, stride = data.shape
    cap = lib.packets_signature_capacity(n, stride)
    d = torch.from_numpy(data.ravel().copy()).cuda()
    dl = torch.from_numpy(lens.view(np.int32).copy()).cuda()
    ws = torch.empty(lib.packets_workspace_size(n, stride), dtype=torch.uint8, device="cuda")
    arrs = [torch.full((cap,), 0x7fffffff, dtype=torch.int32, device="cuda") for _ in range(4)]
    dc = torch.zeros(n, dtype=torch.int32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.extract_offsets_device(d, stride, dl, ws, *arrs, counts=dc, total=tot,
                               stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    t = int(tot.item())
    assert t == counts.sum()
    assert np.array_equal(dc.cpu().numpy().astype(np.uint32), counts)
    for a, e in zip(arrs, (ml, ko, so, mo)):
        assert np.array_equal(a[:t].cpu().numpy().view(np.uint32), e)


def test_verify_packets_fuzzed(lib, oracle):
    data, lens = _fuzzed(oracle, 2000, 203)
    exp, _, counts = oracle.verify_wire_packets(data, data.shape[1], lens, nthreads())
    out, got = lib.verify_packets(data, lens)
    assert np.array_equal(out, exp) and np.array_equal(got, counts)
