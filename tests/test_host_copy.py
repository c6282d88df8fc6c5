"""The library's parallel staging copy (csrc/host_copy.h), built with the
host compiler and run on the CPU: random piece layouts above and below the
parallel threshold, from four caller threads at once."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "solana-perf-libs_gb300", "csrc")


@pytest.mark.parametrize("threads", ["8", "1", "3"])
def test_copy_pool(tmp_path, threads):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "host_copy_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", f"-I{CSRC}", os.path.join(HERE, "native", "host_copy_check.cpp"),
                    "-o", str(exe)], check=True)
    env = dict(os.environ, GB300_CRYPT_COPY_THREADS=threads)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
