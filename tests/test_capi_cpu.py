"""C ABI checks that need no GPU: the library builds, loads, and exports every entry point
declared in include/psoci_gpu.h; without a device, psoci_create fails with a status."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "psoci_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"PSOCI_API\s+[\w\s\*]*?\b(psoci_\w+)\s*\(", txt)))


def test_header_declares_expected_api():
    syms = declared_symbols()
    for s in ["psoci_create", "psoci_destroy", "psoci_set_integrals", "psoci_set_configs", "psoci_build_determinants",
              "psoci_build_hamiltonian", "psoci_get_diag", "psoci_sigma", "psoci_davidson", "psoci_status_str"]:
        assert s in syms


def test_library_exports_all_declared(gpu_lib):
    from psoci_gb300 import build

    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (psoci_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(gpu_lib, s)


def test_python_binding_covers_header():
    from psoci_gb300 import api

    assert set(declared_symbols()) <= set(api.SIGNATURES)


def test_status_strings(gpu_lib):
    for code in range(10):
        assert gpu_lib.psoci_status_str(code)


def test_create_without_device_fails_cleanly(gpu_lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from psoci_gb300 import api

    with pytest.raises(api.PsociError):
        api.Context(0)


def test_null_arguments_rejected(gpu_lib):
    # no context: every entry point must return a status, never crash
    assert gpu_lib.psoci_create(None, None) == 1
    assert gpu_lib.psoci_build_determinants(None) == 1
    assert gpu_lib.psoci_set_integrals(None, 4, None, None, 0.0) == 1
    assert gpu_lib.psoci_sigma(None, 1, None, None, 0) == 1


def test_cpp_host_headers_compile():
    """The C++ class mirrors in include/psoci/ compile against the C ABI."""
    src = os.path.join(ROOT, "psoci_gb300", "host", "driver_splittest.cpp")
    if not os.path.exists(src):
        pytest.skip("C++ host driver not present")
    out = os.path.join(ROOT, "psoci_gb300", "_lib", "test_driver_compile.o")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
