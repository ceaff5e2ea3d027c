"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/phdflux.h declares (no kernel is launched: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

import phd_code_gb300 as pkg
from phd_code_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(phd_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("phd_build", os.path.join(ROOT, "phd-code_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return ctypes.CDLL(b.LIB)


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_declarations(lib):
    assert set(declared()) <= set(_lib.SIGNATURES), set(declared()) - set(_lib.SIGNATURES)


def test_host_only_calls(lib):
    lib.phd_abi_version.restype = ctypes.c_int
    assert lib.phd_abi_version() == 1
    lib.phd_status_string.restype = ctypes.c_char_p
    lib.phd_status_string.argtypes = [ctypes.c_int]
    assert lib.phd_status_string(1) == b"Mass less than zero in flux update"
