"""The C ABI library loads without a GPU and exports every entry point that
include/dpm_gb300.h declares; the ctypes binding declares each of them.
No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dpm_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(dpm\w+)\s*\(", text, flags=re.M)))


def test_header_parses():
    names = declared()
    assert "dpm2d_step" in names and "dpm_serve_step" in names and "dpm2d_step_noalloc" in names
    assert len(names) >= 40


def test_library_exports_header():
    from opencl_dpm_gb300 import abi
    if not os.path.exists(abi.LIB_PATH):
        pytest.skip("library not built")
    lib = ctypes.CDLL(abi.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared()) == set(abi.SIGNATURES), set(declared()) ^ set(abi.SIGNATURES)
    abi.load(strict=True)
    assert abi.load().dpm_version().decode()
