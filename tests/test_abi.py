"""The C-ABI library builds for sm_103a, loads, and exports every function
that include/*.h declares -- and nothing else.  No compute calls: runs
without a GPU."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from conftest import REPO, PKG


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def built_lib():
    import cuda_crypt
    if not os.path.exists(cuda_crypt.LIB_PATH):
        cuda_crypt.build()
    return cuda_crypt.LIB_PATH


def test_headers_declare_reference_abi():
    names = declared_functions()
    reference_abi = {
        "ed25519_init", "ed25519_set_verbose", "ed25519_verify_many", "ed25519_sign_many", "poh_verify_many",
        "poh_verify_many_set_verbose", "cuda_host_register", "cuda_host_unregister", "ed25519_verify",
        "ed25519_sign", "ed25519_create_keypair", "ed25519_create_seed", "ed25519_get_checked_scalar",
        "ed25519_check_packed_ge_small_order", "ed25519_license", "ed25519_free_gpu_mem",
    }
    assert reference_abi <= names, reference_abi - names


def test_library_exports_exactly_the_headers(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = declared_functions()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    exported = {e.split("@")[0] for e in exported}
    assert exported == names, (exported - names, names - exported)


def test_library_is_sm103a(built_lib):
    # the build line pins the architecture; check it in the Makefile the build used
    mk = open(os.path.join(PKG, "Makefile")).read()
    assert "arch=compute_103a,code=sm_103a" in mk


def test_license_string(built_lib):
    lib = ctypes.CDLL(built_lib)
    lib.ed25519_license.restype = ctypes.c_char_p
    assert b"Apache" in lib.ed25519_license()


def test_checked_scalar_host_rule(built_lib):
    """ed25519_get_checked_scalar is a byte test; it needs no GPU."""
    lib = ctypes.CDLL(built_lib)
    out = (ctypes.c_uint8 * 32)()
    ok = bytes(31) + b"\x0f"
    bad = bytes(31) + b"\x10"
    assert lib.ed25519_get_checked_scalar(out, ok) == 0 and bytes(out) == ok
    assert lib.ed25519_get_checked_scalar(out, bad) == 1
