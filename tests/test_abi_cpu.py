"""C ABI checks that need no GPU: the library builds, loads and exports every
entry point include/gca3d.h declares; the header and the binding agree."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gca3d.h")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char)\s*\**\s*(gca3d_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from cuda_3d_gb300 import build

    return build.build()


def test_header_and_binding_agree():
    from cuda_3d_gb300 import native

    assert header_functions() == native.exported_symbols()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gca3d_\w+)", out))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing


def test_library_loads_without_gpu(lib_path):
    from cuda_3d_gb300 import native

    L = native.load(lib_path)
    for name in native.exported_symbols():
        assert getattr(L, name) is not None
    assert L.gca3d_status_string(0) == b"ok"
    assert L.gca3d_status_string(native.ERR_TIMEOUT) == b"device wait timed out"


def test_create_fails_cleanly_without_device(lib_path):
    import ctypes as C

    import torch

    from cuda_3d_gb300 import native

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = native.load(lib_path)
    h = C.c_void_p()
    assert L.gca3d_create(0, None, C.byref(h)) == native.ERR_INVALID_VALUE
    assert not h.value


def test_oracle_builds():
    import oracle as O

    assert os.path.exists(O.build())


def test_kernel_sources_are_sm103a_only():
    """every CUDA translation unit is built with exactly one -gencode (sm_103a)"""
    from cuda_3d_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
