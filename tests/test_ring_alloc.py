"""The served loop's ring allocator (csrc/ring_alloc.h: arrival-order
allocation from a circular buffer, release in any order), built with the host
compiler and run on the CPU: random allocation and release sequences keep
live ranges disjoint, aligned and inside the buffer, and all space returns."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "solana-perf-libs_gb300", "csrc")


def test_ring_alloc(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "ring_alloc_check"
    subprocess.run([cxx, "-O2", "-std=c++17", f"-I{CSRC}", os.path.join(HERE, "native", "ring_alloc_check.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
