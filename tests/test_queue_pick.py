"""The C ABI's choice of GPU and queue per call (csrc/queue_pick.h, used by
acquire() in csrc/crypt_api.cu), built with the host compiler and run on the
CPU with faked device counts of 0 to 8: successive calls rotate the GPUs as
the reference's pool does (src/cuda-ecc-ed25519/gpu_ctx.cu:56-61),
concurrent callers spread over GPUs and queues, and callers beyond the
queue count wait their turn without sharing a queue."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "solana-perf-libs_gb300", "csrc")


def test_queue_pick(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "queue_pick_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", f"-I{CSRC}",
                    os.path.join(HERE, "native", "queue_pick_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
