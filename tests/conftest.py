import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "solana-perf-libs_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

# as the library does when it creates the CUDA context itself: enough hardware
# work queues that unrelated streams do not serialise (torch may create the
# context first)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import get_oracle
    return get_oracle()


@pytest.fixture(scope="session")
def ref():
    from oracle.oracle import build_ref, get_ref
    try:
        build_ref()
    except Exception:
        pass
    r = get_ref()
    if r is None:
        pytest.skip("the reference's own code is not available on this machine")
    return r


@pytest.fixture(scope="session")
def lib():
    import cuda_crypt
    if not os.path.exists(cuda_crypt.LIB_PATH):
        cuda_crypt.build()
    L = cuda_crypt.get_lib()
    assert L.init(), "ed25519_init() found no usable GPU"
    return L


@pytest.fixture(scope="session")
def golden_poh():
    with open(os.path.join(GOLDEN, "poh_332.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_ed():
    with open(os.path.join(GOLDEN, "ed25519_ref.json")) as f:
        return json.load(f)


def nthreads():
    return os.cpu_count() or 1
