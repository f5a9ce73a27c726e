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


def test_python_signatures_match_prototypes():
    # the ctypes table against the header: argument count and each type's
    # size and kind (pointers as c_void_p, POINTER(...) or c_char_p)
    from glagpu import _lib
    from test_julia_glue import prototypes
    scalars = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "size_t": ctypes.c_size_t,
               "double": ctypes.c_double, "float": ctypes.c_float, "char": ctypes.c_char}
    for name, (cret, ctypes_) in prototypes().items():
        args, ret = _lib.SIGNATURES[name]
        assert len(args) == len(ctypes_), name
        for c, t in zip(ctypes_ + [cret], list(args) + [ret]):
            c = c.replace("const ", "").strip()
            if c.endswith("*") or c == "gla_plan_t":
                assert t in (ctypes.c_void_p, ctypes.c_char_p) or t.__name__.startswith("LP_"), (name, c, t)
            else:
                assert ctypes.sizeof(t) == ctypes.sizeof(scalars[c]), (name, c, t)
                assert (t in (ctypes.c_float, ctypes.c_double)) == (c in ("float", "double")), (name, c, t)


def test_host_only_calls(lib):
    lib.gla_version.restype = ctypes.c_int
    assert lib.gla_version() == 100
    lib.gla_status_string.restype = ctypes.c_char_p
    lib.gla_status_string.argtypes = [ctypes.c_int]
    assert lib.gla_status_string(0) == b"success"
    assert b"argument 3" in lib.gla_status_string(-3)


def test_header_is_plain_c_and_links(lib, tmp_path):
    # the boundary is a C ABI: the header compiles as strict C99 and a C
    # program that takes the address of every declared entry point links
    # against the library and runs its host-only calls
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    syms = header_symbols()
    src = tmp_path / "abi.c"
    src.write_text('#include "glagpu.h"\n#include <stdio.h>\n'
                   "typedef void (*fn)(void);\n"
                   "static const fn table[] = {" + ", ".join(f"(fn){s}" for s in syms) + "};\n"
                   "int main(void) {\n"
                   "  printf(\"%d %d\\n\", gla_version(), (int)(sizeof(table) / sizeof(table[0])));\n"
                   "  return 0;\n}\n")
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib._name)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", libdir, "-lglagpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.split() == ["100", str(len(syms))]


def test_autotune_table_file_roundtrip(lib, tmp_path):
    # host-only: the table's text format, validation of loaded lines, save
    lib.gla_autotune_load.argtypes = [ctypes.c_char_p]
    lib.gla_autotune_save.argtypes = [ctypes.c_char_p]
    assert lib.gla_autotune_clear() == 0
    src = tmp_path / "tune.txt"
    src.write_text("# comment\n"
                   "0 V 7 9 2 16 1.5 3.25\n"
                   "1 N 0 4 4 32 0.1 0.2\n"
                   "1 V 3 2 3 8 0.1 0.2\n"      # tri_mult 3: rejected
                   "0 V 2 1 1 64 0.1 0.2\n"     # 64 lanes: rejected
                   "garbage line\n")
    assert lib.gla_autotune_load(str(src).encode()) == 2
    out = tmp_path / "out.txt"
    assert lib.gla_autotune_save(str(out).encode()) == 0
    rows = [l.split() for l in out.read_text().splitlines() if not l.startswith("#")]
    assert sorted((r[0], r[1], r[2], r[3], r[4], r[5]) for r in rows) == \
        [("0", "V", "7", "9", "2", "16"), ("1", "N", "0", "4", "4", "32")]
    assert lib.gla_autotune_load(str(tmp_path / "missing.txt").encode()) < 0
    assert lib.gla_autotune_clear() == 0
