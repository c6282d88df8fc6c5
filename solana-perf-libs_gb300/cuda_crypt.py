"""Python binding of libcuda-crypt.so (the GB300 Ed25519 / PoH library).

Mirrors the reference's C interface (src/cuda-ecc-ed25519/ed25519.h,
src/cuda-poh-verify/poh_verify.cu) one function per export, with the same
argument meaning, over numpy buffers; plus the device-pointer forms for
buffers already resident on the GPU (torch tensors).  There is no CPU path:
loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcuda-crypt.so")

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class GpuElems(ctypes.Structure):
    """gpu_Elems (reference ed25519.h:35-38)."""
    _fields_ = [("elems", _u8p), ("num", ctypes.c_uint32)]


class SigJob(ctypes.Structure):
    """gb300_sig_job: one verify (kind 0) or sign (kind 1) job of a ragged batch."""
    _fields_ = [("packets", _u8p), ("packets_len", ctypes.c_uint64), ("message_lens", _u32p),
                ("public_key_offsets", _u32p), ("key_offsets", _u32p), ("message_start_offsets", _u32p),
                ("num", ctypes.c_uint32), ("kind", ctypes.c_uint32), ("out", _u8p)]


JOB_VERIFY, JOB_SIGN = 0, 1


def build(jobs: int = 8) -> str:
    """Compile libcuda-crypt.so for sm_103a in place (make, parallel TUs)."""
    subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs}", "libcuda-crypt.so"], check=True)
    return LIB_PATH


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class SigPackets:
    """A signature batch in the reference's layout: packets of `message_size`
    bytes back to back (one gpu_Elems run per entry of `batches`), and four
    uint32 arrays with one entry per signature."""
    batches: list            # list of np.uint8 arrays, each (num * message_size,)
    message_size: int
    message_lens: np.ndarray
    public_key_offsets: np.ndarray
    signature_offsets: np.ndarray        # private-key offsets when signing
    message_start_offsets: np.ndarray

    @property
    def total_signatures(self) -> int:
        return int(len(self.message_lens))

    @property
    def total_packets(self) -> int:
        return int(sum(len(b) for b in self.batches) // max(1, self.message_size))

    def concatenated(self) -> np.ndarray:
        return np.concatenate(self.batches) if len(self.batches) > 1 else self.batches[0]


class CudaCrypt:
    """ctypes view of libcuda-crypt.so."""

    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise RuntimeError(f"libcuda-crypt.so not built ({path}); run cuda_crypt.build()")
        self.path = path
        L = self.lib = ctypes.CDLL(path)
        L.ed25519_init.restype = ctypes.c_bool
        L.ed25519_set_verbose.argtypes = [ctypes.c_bool]
        sig_many = [ctypes.POINTER(GpuElems), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                    _u32p, _u32p, _u32p, _u32p, _u8p, ctypes.c_uint8]
        L.ed25519_verify_many.argtypes = sig_many
        L.ed25519_verify_many.restype = None
        L.ed25519_sign_many.argtypes = sig_many
        L.ed25519_sign_many.restype = None
        L.poh_verify_many.argtypes = [_u8p, _u64p, ctypes.c_size_t, ctypes.c_uint8]
        L.poh_verify_many.restype = ctypes.c_int
        L.poh_verify_many_set_verbose.argtypes = [ctypes.c_bool]
        L.ed25519_verify.argtypes = [_u8p, _u8p, ctypes.c_uint32, _u8p]
        L.ed25519_verify.restype = ctypes.c_int
        L.ed25519_sign.argtypes = [_u8p, _u8p, ctypes.c_size_t, _u8p, _u8p]
        L.ed25519_create_keypair.argtypes = [_u8p, _u8p, _u8p]
        L.ed25519_create_seed.argtypes = [_u8p]
        L.ed25519_get_checked_scalar.argtypes = [_u8p, _u8p]
        L.ed25519_check_packed_ge_small_order.argtypes = [_u8p]
        L.ed25519_license.restype = ctypes.c_char_p
        L.cuda_host_register.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint]
        L.cuda_host_register.restype = ctypes.c_int
        L.cuda_host_unregister.argtypes = [ctypes.c_void_p]
        L.cuda_host_unregister.restype = ctypes.c_int
        L.gb300_crypt_last_error.restype = ctypes.c_int
        dev_sig = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        L.gb300_ed25519_verify_device.argtypes = dev_sig
        L.gb300_ed25519_sign_device.argtypes = dev_sig
        L.gb300_ed25519_keypair_device.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_uint32, ctypes.c_void_p]
        L.gb300_poh_verify_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        L.gb300_ed25519_create_keypairs.argtypes = [_u8p, _u8p, _u8p, ctypes.c_uint32]
        L.gb300_ed25519_batch.argtypes = [ctypes.POINTER(SigJob), ctypes.c_uint32]
        L.gb300_ed25519_batch_device.argtypes = [ctypes.c_void_p, ctypes.c_uint64] + [ctypes.c_void_p] * 4 + \
            [ctypes.c_uint32, ctypes.c_void_p] + [ctypes.c_void_p] * 4 + [ctypes.c_uint32, ctypes.c_void_p,
                                                                        ctypes.c_void_p, ctypes.c_void_p]
        L.gb300_poh_verify_batch.argtypes = [_u8p, _u64p, ctypes.c_size_t]
        L.gb300_poh_batch_workspace_size.argtypes = [ctypes.c_uint64]
        L.gb300_poh_batch_workspace_size.restype = ctypes.c_size_t
        L.gb300_poh_verify_batch_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                    ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        L.gb300_crypt_tuning.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.gb300_poh_verify_batch_shape.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_void_p]
        L.gb300_poh_verify_batch_shape.restype = ctypes.c_int
        L.gb300_packets_workspace_size.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.gb300_packets_workspace_size.restype = ctypes.c_size_t
        L.gb300_packets_signature_capacity.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.gb300_packets_signature_capacity.restype = ctypes.c_uint64
        L.gb300_packets_extract_offsets_device.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t] + \
            [ctypes.c_void_p] * 7
        L.gb300_packets_extract_offsets_device.restype = ctypes.c_int
        L.gb300_ed25519_verify_packets_device.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.gb300_ed25519_verify_packets_device.restype = ctypes.c_int
        L.gb300_ed25519_verify_packets.argtypes = [ctypes.POINTER(GpuElems), ctypes.c_uint32, ctypes.c_uint32,
                                                   _u32p, _u8p, _u32p]
        L.gb300_ed25519_verify_packets.restype = ctypes.c_int
        L.gb300_ed25519_verify_device_form.argtypes = [ctypes.c_void_p, ctypes.c_uint64] + [ctypes.c_void_p] * 4 + \
            [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.gb300_ed25519_verify_device_form.restype = ctypes.c_int
        L.gb300_diag_half_scalars.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        L.gb300_diag_half_scalars.restype = ctypes.c_int

    # ---- reference entry points ------------------------------------------
    def init(self) -> bool:
        return bool(self.lib.ed25519_init())

    def set_verbose(self, v: bool) -> None:
        self.lib.ed25519_set_verbose(bool(v))

    def last_error(self) -> int:
        return int(self.lib.gb300_crypt_last_error())

    def _elems(self, batches: Sequence[np.ndarray], message_size: int):
        arr = (GpuElems * max(1, len(batches)))()
        for i, b in enumerate(batches):
            arr[i].elems = _p(b, _u8p)
            arr[i].num = len(b) // message_size if message_size else 0
        return arr

    def _sig_call(self, fn, sp: SigPackets, out: np.ndarray, use_non_default_stream: int):
        batches = [np.ascontiguousarray(b, dtype=np.uint8) for b in sp.batches]
        arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
                (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)]
        elems = self._elems(batches, sp.message_size)
        total_packets = sum(len(b) // sp.message_size for b in batches) if sp.message_size else 0
        fn(elems, len(batches), sp.message_size, total_packets, len(arrs[0]), *[_p(a, _u32p) for a in arrs],
           _p(out, _u8p), use_non_default_stream)
        return out

    def verify_many(self, sp: SigPackets, use_non_default_stream: int = 1) -> np.ndarray:
        out = np.zeros(sp.total_signatures, dtype=np.uint8)
        return self._sig_call(self.lib.ed25519_verify_many, sp, out, use_non_default_stream)

    def sign_many(self, sp: SigPackets, use_non_default_stream: int = 1) -> np.ndarray:
        out = np.zeros((sp.total_signatures, 64), dtype=np.uint8)
        return self._sig_call(self.lib.ed25519_sign_many, sp, out, use_non_default_stream)

    def poh_verify_many(self, hashes: np.ndarray, num_hashes, use_non_default_stream: int = 1) -> int:
        """In place on `hashes` (uint8, n*32), like the reference."""
        assert hashes.dtype == np.uint8 and hashes.flags["C_CONTIGUOUS"]
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        return int(self.lib.poh_verify_many(_p(hashes, _u8p), _p(nh, _u64p), len(nh), use_non_default_stream))

    def verify(self, sig: bytes, msg: bytes, pk: bytes) -> int:
        return int(self.lib.ed25519_verify(_buf(sig), _buf(msg), len(msg), _buf(pk)))

    def sign(self, msg: bytes, pk: bytes, sk: bytes) -> bytes:
        out = (ctypes.c_uint8 * 64)()
        self.lib.ed25519_sign(out, _buf(msg), len(msg), _buf(pk), _buf(sk))
        return bytes(out)

    def create_keypair(self, seed: bytes):
        pk = (ctypes.c_uint8 * 32)()
        sk = (ctypes.c_uint8 * 64)()
        self.lib.ed25519_create_keypair(pk, sk, _buf(seed))
        return bytes(pk), bytes(sk)

    def create_keypairs(self, seeds: np.ndarray):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint8).reshape(-1, 32)
        n = len(seeds)
        pk = np.zeros((n, 32), dtype=np.uint8)
        sk = np.zeros((n, 64), dtype=np.uint8)
        rc = self.lib.gb300_ed25519_create_keypairs(_p(seeds, _u8p), _p(pk, _u8p), _p(sk, _u8p), n)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_create_keypairs failed: cudaError {rc}")
        return pk, sk

    def get_checked_scalar(self, s: bytes) -> int:
        out = (ctypes.c_uint8 * 32)()
        return int(self.lib.ed25519_get_checked_scalar(out, _buf(s)))

    def check_packed_ge_small_order(self, p: bytes) -> int:
        return int(self.lib.ed25519_check_packed_ge_small_order(_buf(p)))

    def license(self) -> str:
        return self.lib.ed25519_license().decode()

    def host_register(self, arr: np.ndarray, flags: int = 0) -> int:
        return int(self.lib.cuda_host_register(arr.ctypes.data, arr.nbytes, flags))

    def host_unregister(self, arr: np.ndarray) -> int:
        return int(self.lib.cuda_host_unregister(arr.ctypes.data))

    # ---- ragged batches in one persistent launch -----------------------------
    def ed25519_batch(self, jobs) -> list:
        """jobs: list of (SigPackets, kind).  Returns one output array per job
        (verdicts for kind 0, (n, 64) signatures for kind 1)."""
        return self.ed25519_batch_run(self.ed25519_batch_prepare(jobs))

    def ed25519_batch_run(self, prepared) -> list:
        """gb300_ed25519_batch on arguments from ed25519_batch_prepare (the
        call alone, as a compiled caller makes it); returns the outputs."""
        arr, n, _, outs = prepared
        rc = self.lib.gb300_ed25519_batch(arr, n)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_batch: cudaError {rc}")
        return outs

    def ed25519_batch_prepare(self, jobs):
        """The gb300_sig_job array for `jobs`, the arrays it points to and
        the output arrays it fills."""
        keep, outs = [], []
        arr = (SigJob * max(1, len(jobs)))()
        for k, (sp, kind) in enumerate(jobs):
            pk = np.ascontiguousarray(sp.concatenated(), dtype=np.uint8)
            arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
                    (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)]
            n = len(arrs[0])
            out = np.zeros(n if kind == JOB_VERIFY else (n, 64), dtype=np.uint8)
            keep += [pk] + arrs
            outs.append(out)
            j = arr[k]
            j.packets = _p(pk, _u8p)
            j.packets_len = pk.nbytes
            j.message_lens, j.public_key_offsets, j.key_offsets, j.message_start_offsets = \
                [_p(a, _u32p) for a in arrs]
            j.num, j.kind, j.out = n, kind, _p(out, _u8p)
        return arr, len(jobs), keep, outs

    def poh_verify_batch(self, hashes: np.ndarray, num_hashes) -> int:
        """In place on `hashes` (uint8, n*32), like poh_verify_many."""
        assert hashes.dtype == np.uint8 and hashes.flags["C_CONTIGUOUS"]
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        return int(self.lib.gb300_poh_verify_batch(_p(hashes, _u8p), _p(nh, _u64p), len(nh)))

    def poh_batch_workspace_size(self, n: int) -> int:
        return int(self.lib.gb300_poh_batch_workspace_size(n))

    def poh_verify_batch_device(self, hashes, num_hashes, workspace, stream=0) -> None:
        rc = self.lib.gb300_poh_verify_batch_device(hashes.data_ptr(), num_hashes.data_ptr(), num_hashes.numel(),
                                                    workspace.data_ptr(), workspace.numel() * workspace.element_size(),
                                                    stream)
        if rc != 0:
            raise RuntimeError(f"gb300_poh_verify_batch_device: cudaError {rc}")

    POH_SINGLE, POH_PACKED_SINGLE, POH_PAIR, POH_PACKED_PAIR, POH_PAIR_DIRECT, POH_AUTO = 0, 1, 2, 3, 4, 5

    def poh_verify_batch_shape(self, hashes, num_hashes, workspace, warps, form, stream=0) -> None:
        """Device PoH batch with a forced persistent launch shape (diagnostic);
        form: POH_SINGLE, POH_PACKED_SINGLE, POH_PAIR, POH_PACKED_PAIR, POH_PAIR_DIRECT or POH_AUTO."""
        rc = self.lib.gb300_poh_verify_batch_shape(hashes.data_ptr(), num_hashes.data_ptr(), num_hashes.numel(),
                                                   workspace.data_ptr(), workspace.numel() * workspace.element_size(),
                                                   warps, form, stream)
        if rc != 0:
            raise RuntimeError(f"gb300_poh_verify_batch_shape: cudaError {rc}")

    # ---- Solana ledger entries: PoH chains with transaction mixins ----
    def _entries_types(self):
        L = self.lib
        if getattr(self, "_entries_ready", False):
            return L
        L.gb300_poh_entries_workspace_size.argtypes = [ctypes.c_uint64]
        L.gb300_poh_entries_workspace_size.restype = ctypes.c_size_t
        L.gb300_poh_verify_entries.argtypes = [_u8p, _u64p, _u8p, _u8p, _u8p, ctypes.c_size_t, _u8p]
        L.gb300_poh_verify_entries.restype = ctypes.c_int
        L.gb300_poh_verify_entries_device.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_uint64] + \
            [ctypes.c_void_p] * 3 + [ctypes.c_size_t, ctypes.c_void_p]
        L.gb300_poh_verify_entries_device.restype = ctypes.c_int
        L.gb300_poh_record.argtypes = [_u8p, ctypes.c_size_t, _u64p, _u64p, _u8p, _u8p, _u8p]
        L.gb300_poh_record.restype = ctypes.c_int
        L.gb300_poh_record_device.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64] + \
            [ctypes.c_void_p] * 5
        L.gb300_poh_record_device.restype = ctypes.c_int
        self._entries_ready = True
        return L

    def poh_entries_workspace_size(self, n: int) -> int:
        return int(self._entries_types().gb300_poh_entries_workspace_size(n))

    def poh_verify_entries(self, start, num_hashes, mixins, has_mixin, expected) -> np.ndarray:
        """ok per entry (host form); 32-byte arrays as (n, 32) uint8."""
        L = self._entries_types()
        st = np.ascontiguousarray(start, dtype=np.uint8).reshape(-1, 32)
        n = len(st)
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        mx = np.ascontiguousarray(mixins, dtype=np.uint8).reshape(-1, 32)
        hm = np.ascontiguousarray(has_mixin, dtype=np.uint8)
        ex = np.ascontiguousarray(expected, dtype=np.uint8).reshape(-1, 32)
        ok = np.zeros(n, dtype=np.uint8)
        rc = L.gb300_poh_verify_entries(_p(st, _u8p), _p(nh, _u64p), _p(mx, _u8p), _p(hm, _u8p), _p(ex, _u8p), n,
                                        _p(ok, _u8p))
        if rc != 0:
            raise RuntimeError(f"gb300_poh_verify_entries: cudaError {rc}")
        return ok

    def poh_verify_entries_device(self, start, num_hashes, mixins, has_mixin, expected, ok, out_hashes, workspace,
                                  stream=0) -> None:
        L = self._entries_types()
        rc = L.gb300_poh_verify_entries_device(start.data_ptr(), num_hashes.data_ptr(), mixins.data_ptr(),
                                               has_mixin.data_ptr(), expected.data_ptr(), num_hashes.numel(),
                                               ok.data_ptr(), out_hashes.data_ptr() if out_hashes is not None else None,
                                               workspace.data_ptr(), workspace.numel() * workspace.element_size(),
                                               stream)
        if rc != 0:
            raise RuntimeError(f"gb300_poh_verify_entries_device: cudaError {rc}")

    def poh_record(self, start, first, num_hashes, mixins, has_mixin):
        """(entry hashes, last hash per chain) (host form); chain c runs
        entries first[c] .. first[c + 1] - 1."""
        L = self._entries_types()
        h = np.array(start, dtype=np.uint8, copy=True).reshape(-1, 32)
        fi = np.ascontiguousarray(first, dtype=np.uint64)
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        mx = np.ascontiguousarray(mixins, dtype=np.uint8).reshape(-1, 32)
        hm = np.ascontiguousarray(has_mixin, dtype=np.uint8)
        out = np.zeros((max(1, len(nh)), 32), dtype=np.uint8)
        rc = L.gb300_poh_record(_p(h, _u8p), len(h), _p(fi, _u64p), _p(nh, _u64p), _p(mx, _u8p), _p(hm, _u8p),
                                _p(out, _u8p))
        if rc != 0:
            raise RuntimeError(f"gb300_poh_record: cudaError {rc}")
        return out[:len(nh)], h

    def poh_record_device(self, hashes, first, num_hashes, mixins, has_mixin, entry_hashes, stream=0) -> None:
        L = self._entries_types()
        rc = L.gb300_poh_record_device(hashes.data_ptr(), first.numel() - 1, first.data_ptr(), num_hashes.numel(),
                                       num_hashes.data_ptr(), mixins.data_ptr(), has_mixin.data_ptr(),
                                       entry_hashes.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_poh_record_device: cudaError {rc}")

    # ---- Solana wire-format packets (gb300_packets.h) ----
    def packets_workspace_size(self, n: int, stride: int) -> int:
        return int(self.lib.gb300_packets_workspace_size(n, stride))

    def packets_signature_capacity(self, n: int, stride: int) -> int:
        return int(self.lib.gb300_packets_signature_capacity(n, stride))

    def verify_packets(self, data: np.ndarray, lens, batches: int = 1):
        """Host form.  `data`: (n, stride) uint8 packet slots, split into
        `batches` gpu_Elems runs; returns (packet verdicts, signatures per
        packet)."""
        assert data.dtype == np.uint8 and data.ndim == 2 and data.flags["C_CONTIGUOUS"]
        n, stride = data.shape
        lens = np.ascontiguousarray(lens, dtype=np.uint32)
        cuts = np.linspace(0, n, batches + 1).astype(int)
        elems = (GpuElems * batches)()
        for i in range(batches):
            elems[i].elems = _p(data[cuts[i]:], _u8p) if cuts[i] < n else None
            elems[i].num = int(cuts[i + 1] - cuts[i])
        out = np.zeros(n, dtype=np.uint8)
        counts = np.zeros(n, dtype=np.uint32)
        rc = self.lib.gb300_ed25519_verify_packets(elems, batches, stride, _p(lens, _u32p), _p(out, _u8p),
                                                   _p(counts, _u32p))
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_verify_packets: cudaError {rc}")
        return out, counts

    def verify_packets_device(self, data, stride, lens, workspace, out, counts=None, stream=0) -> None:
        rc = self.lib.gb300_ed25519_verify_packets_device(
            data.data_ptr(), stride, lens.numel(), lens.data_ptr(), workspace.data_ptr(),
            workspace.numel() * workspace.element_size(), out.data_ptr(),
            counts.data_ptr() if counts is not None else None, stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_verify_packets_device: cudaError {rc}")

    def extract_offsets_device(self, data, stride, lens, workspace, message_lens, key_offsets, sig_offsets,
                               msg_offsets, counts=None, total=None, stream=0) -> None:
        rc = self.lib.gb300_packets_extract_offsets_device(
            data.data_ptr(), stride, lens.numel(), lens.data_ptr(), workspace.data_ptr(),
            workspace.numel() * workspace.element_size(), message_lens.data_ptr(), key_offsets.data_ptr(),
            sig_offsets.data_ptr(), msg_offsets.data_ptr(), counts.data_ptr() if counts is not None else None,
            total.data_ptr() if total is not None else None, stream)
        if rc != 0:
            raise RuntimeError(f"gb300_packets_extract_offsets_device: cudaError {rc}")

    def ed25519_batch_device(self, packets, v, v_out, s, s_out, queue_word, stream=0) -> None:
        """v / s: 4 device int32 tensors (lens, pubkey, sig-or-privkey, message offsets)."""
        nv = v[0].numel() if v else 0
        ns = s[0].numel() if s else 0
        vp = [t.data_ptr() for t in v] if v else [0, 0, 0, 0]
        spp = [t.data_ptr() for t in s] if s else [0, 0, 0, 0]
        rc = self.lib.gb300_ed25519_batch_device(packets.data_ptr(), packets.numel(), *vp, nv,
                                                 v_out.data_ptr() if nv else 0, *spp, ns,
                                                 s_out.data_ptr() if ns else 0, queue_word.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_batch_device: cudaError {rc}")

    def tuning(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(1024)
        n = self.lib.gb300_crypt_tuning(buf, 1024)
        return json.loads(buf.value[:n].decode()) if n else {}

    # ---- device-pointer forms (torch tensors on the GPU) -------------------
    def verify_device(self, packets, message_lens, public_key_offsets, signature_offsets, message_start_offsets,
                      out, stream=0) -> None:
        rc = self.lib.gb300_ed25519_verify_device(
            packets.data_ptr(), packets.numel(), message_lens.data_ptr(), public_key_offsets.data_ptr(),
            signature_offsets.data_ptr(), message_start_offsets.data_ptr(), message_lens.numel(),
            out.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_verify_device: cudaError {rc}")

    VERIFY_SINGLE, VERIFY_QUAD, VERIFY_SINGLE_W4, VERIFY_SINGLE_W5, VERIFY_TRIO, VERIFY_STAGED, VERIFY_HALF = 0, 1, 2, 3, 4, 5, 6

    def verify_device_form(self, packets, message_lens, public_key_offsets, signature_offsets,
                           message_start_offsets, out, form, stream=0) -> None:
        """verify_device with the kernel form forced (diagnostic)."""
        rc = self.lib.gb300_ed25519_verify_device_form(
            packets.data_ptr(), packets.numel(), message_lens.data_ptr(), public_key_offsets.data_ptr(),
            signature_offsets.data_ptr(), message_start_offsets.data_ptr(), message_lens.numel(),
            out.data_ptr(), form, stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_verify_device_form: cudaError {rc}")

    def half_scalars_device(self, h, out, stream=0) -> None:
        """The three-warp verify form's half-size scalars of h (uint32 tensor
        [n, 8]) into out (uint32 tensor [n, 18]) (diagnostic)."""
        rc = self.lib.gb300_diag_half_scalars(h.data_ptr(), h.shape[0], out.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_diag_half_scalars: cudaError {rc}")

    def sign_device(self, packets, message_lens, public_key_offsets, private_key_offsets, message_start_offsets,
                    out, stream=0) -> None:
        rc = self.lib.gb300_ed25519_sign_device(
            packets.data_ptr(), packets.numel(), message_lens.data_ptr(), public_key_offsets.data_ptr(),
            private_key_offsets.data_ptr(), message_start_offsets.data_ptr(), message_lens.numel(),
            out.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_sign_device: cudaError {rc}")

    def keypair_device(self, seeds, pk, sk, stream=0) -> None:
        rc = self.lib.gb300_ed25519_keypair_device(seeds.data_ptr(), pk.data_ptr(), sk.data_ptr(),
                                                   seeds.numel() // 32, stream)
        if rc != 0:
            raise RuntimeError(f"gb300_ed25519_keypair_device: cudaError {rc}")

    def poh_verify_device(self, hashes, num_hashes, stream=0) -> None:
        rc = self.lib.gb300_poh_verify_device(hashes.data_ptr(), num_hashes.data_ptr(), num_hashes.numel(), stream)
        if rc != 0:
            raise RuntimeError(f"gb300_poh_verify_device: cudaError {rc}")


class ServerConfig(ctypes.Structure):
    _fields_ = [("device_memory_cap", ctypes.c_uint64), ("sig_slots", ctypes.c_uint32),
                ("poh_slots", ctypes.c_uint32), ("max_items_per_launch", ctypes.c_uint32),
                ("sig_mode", ctypes.c_uint32)]

SIG_SERVICE, SIG_SLOTS = 0, 1       # ServerConfig.sig_mode


class Server:
    """The served request loop (include/gb300_serve.h) on the current GPU."""

    def __init__(self, lib: "CudaCrypt", device_memory_cap: int = 0, sig_slots: int = 0, poh_slots: int = 0,
                 max_items_per_launch: int = 0, sig_mode: int = SIG_SERVICE):
        L = self.L = lib.lib
        L.gb300_server_create.argtypes = [ctypes.POINTER(ServerConfig)]
        L.gb300_server_create.restype = ctypes.c_void_p
        L.gb300_server_destroy.argtypes = [ctypes.c_void_p]
        L.gb300_server_submit_sigs.argtypes = [ctypes.c_void_p, ctypes.POINTER(SigJob)]
        L.gb300_server_submit_sigs.restype = ctypes.c_uint64
        L.gb300_server_submit_poh.argtypes = [ctypes.c_void_p, _u8p, _u64p, ctypes.c_size_t]
        L.gb300_server_submit_poh.restype = ctypes.c_uint64
        L.gb300_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.gb300_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int]
        L.gb300_server_release.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.gb300_server_stats.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
        L.gb300_server_times.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int64),
                                         ctypes.POINTER(ctypes.c_int64)]
        L.gb300_server_submit_packets.argtypes = [ctypes.c_void_p, ctypes.POINTER(GpuElems), ctypes.c_uint32,
                                                  ctypes.c_uint32, _u32p, _u8p, _u32p]
        L.gb300_server_submit_packets.restype = ctypes.c_uint64
        L.gb300_server_trace.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
        L.gb300_server_trace.restype = ctypes.c_int
        cfg = ServerConfig(device_memory_cap, sig_slots, poh_slots, max_items_per_launch, sig_mode)
        self.h = L.gb300_server_create(ctypes.byref(cfg))
        if not self.h:
            raise RuntimeError("gb300_server_create failed")
        self._keep = {}

    def submit_sigs(self, sp: SigPackets, kind: int, out: np.ndarray | None = None):
        """Queues one verify/sign job; returns (ticket, out).  `out` is filled
        when the ticket completes."""
        pk = np.ascontiguousarray(sp.concatenated(), dtype=np.uint8)
        arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in
                (sp.message_lens, sp.public_key_offsets, sp.signature_offsets, sp.message_start_offsets)]
        n = len(arrs[0])
        if out is None:
            out = np.zeros(n if kind == JOB_VERIFY else (n, 64), dtype=np.uint8)
        j = SigJob(_p(pk, _u8p), pk.nbytes, *[_p(a, _u32p) for a in arrs], n, kind, _p(out, _u8p))
        t = self.L.gb300_server_submit_sigs(self.h, ctypes.byref(j))
        if t:
            self._keep[t] = (pk, arrs, out, j)
        return t, out

    def submit_packets(self, data: np.ndarray, lens, batches: int = 1, counts: bool = True):
        """Queues wire-format packets: `data` (n, stride) uint8 slots split
        into `batches` gpu_Elems runs.  Returns (ticket, packet verdicts,
        signatures per packet or None), filled when the ticket completes."""
        assert data.dtype == np.uint8 and data.ndim == 2 and data.flags["C_CONTIGUOUS"]
        n, stride = data.shape
        lens = np.ascontiguousarray(lens, dtype=np.uint32)
        elems = (GpuElems * batches)()
        if batches == 1:
            elems[0].elems = _p(data, _u8p)
            elems[0].num = n
        else:
            cuts = np.linspace(0, n, batches + 1).astype(int)
            for i in range(batches):
                elems[i].elems = _p(data[cuts[i]:], _u8p) if cuts[i] < n else None
                elems[i].num = int(cuts[i + 1] - cuts[i])
        out = np.zeros(n, dtype=np.uint8)
        cnt = np.zeros(n, dtype=np.uint32) if counts else None
        t = self.L.gb300_server_submit_packets(self.h, elems, batches, stride, _p(lens, _u32p), _p(out, _u8p),
                                               _p(cnt, _u32p) if counts else None)
        if t:
            self._keep[t] = (data, lens, out, cnt)
        return t, out, cnt

    def submit_poh(self, hashes: np.ndarray, num_hashes):
        nh = np.ascontiguousarray(num_hashes, dtype=np.uint64)
        assert hashes.dtype == np.uint8 and hashes.flags["C_CONTIGUOUS"]
        t = self.L.gb300_server_submit_poh(self.h, _p(hashes, _u8p), _p(nh, _u64p), len(nh))
        if t:
            self._keep[t] = (hashes, nh)
        return t

    def poll(self, ticket: int) -> int:
        return int(self.L.gb300_server_poll(self.h, ticket))

    def wait(self, ticket: int, timeout_ms: int = -1, release: bool = True) -> int:
        rc = int(self.L.gb300_server_wait(self.h, ticket, timeout_ms))
        if rc != 0 and release:
            self.release(ticket)
        return rc

    def release(self, ticket: int) -> None:
        self.L.gb300_server_release(self.h, ticket)
        self._keep.pop(ticket, None)

    def latency_s(self, ticket: int):
        """Completion minus submission time (seconds), None while pending."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        rc = self.L.gb300_server_times(self.h, ticket, ctypes.byref(a), ctypes.byref(b))
        return (b.value - a.value) * 1e-9 if rc == 1 else None

    def times_ns(self, ticket: int):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self.L.gb300_server_times(self.h, ticket, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def stats(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(1024)
        n = self.L.gb300_server_stats(self.h, buf, 1024)
        return json.loads(buf.value[:n].decode()) if n else {}

    def trace(self) -> list:
        """Recent launches: [kind, requests, items, admitted_ns, enqueued_ns,
        completed_ns, copy_in_ms, kernels_ms, copy_out_ms] each."""
        import json
        buf = ctypes.create_string_buffer(1 << 22)
        n = self.L.gb300_server_trace(self.h, buf, len(buf))
        return json.loads(buf.value[:n].decode()) if n else []

    def close(self) -> None:
        if self.h:
            self.L.gb300_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _buf(b) -> ctypes.Array:
    b = bytes(b)
    return (ctypes.c_uint8 * max(1, len(b))).from_buffer_copy(b if b else b"\0")


_lib = None


def get_lib() -> CudaCrypt:
    global _lib
    if _lib is None:
        _lib = CudaCrypt()
    return _lib
