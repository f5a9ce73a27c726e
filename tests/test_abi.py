"""The C-ABI library builds for sm_103a, loads, and exports every symbol
include/glagpu.h declares (host-only calls, no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "glagpu.h")).read()
    return sorted(set(re.findall(r"\b(gla_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gla_build", os.path.join(ROOT, "genericlinearalgebra.jl_gb300",
                                                                         "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return ctypes.CDLL(m.build())


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_header():
    from glagpu import _lib
    assert set(_lib.SIGNATURES) == set(header_symbols())


def test_host_only_calls(lib):
    lib.gla_version.restype = ctypes.c_int
    assert lib.gla_version() == 100
    lib.gla_status_string.restype = ctypes.c_char_p
    lib.gla_status_string.argtypes = [ctypes.c_int]
    assert lib.gla_status_string(0) == b"success"
    assert b"argument 3" in lib.gla_status_string(-3)
