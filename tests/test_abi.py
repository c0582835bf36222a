"""The C ABI library loads and exports every symbol include/cfgpu.h declares; the C++
drop-in header compiles.  No compute calls (these run without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "compfinance_gb300", "libcfgpu.so")


def declared():
    txt = open(os.path.join(ROOT, "include", "cfgpu.h")).read()
    return sorted(set(re.findall(r"^int (cf_\w+)\(", txt, re.M)))


def test_header_declares_entry_points():
    names = declared()
    for n in ("cf_create", "cf_value", "cf_aad_risk_one", "cf_aad_risk_aggregate", "cf_aad_risk_multi",
              "cf_dupire_calib", "cf_dupire_superbucket", "cf_put_dupire", "cf_put_barrier"):
        assert n in names


def test_library_exports_every_symbol():
    if not os.path.exists(LIB):
        from compfinance_gb300 import build
        build.build()
    lib = ctypes.CDLL(LIB)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("caller", ["dropin_main.cpp", "objects_main.cpp"])
def test_cpp_dropin_headers_compile(caller):
    src = os.path.join(ROOT, "tests", "cpp", caller)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_last_error_without_context():
    lib = ctypes.CDLL(LIB)
    h = ctypes.c_void_p()
    # a null output pointer is rejected before any device call
    assert lib.cf_create(0, None) == -1
    buf = ctypes.create_string_buffer(256)
    assert lib.cf_last_error(buf, ctypes.c_size_t(256)) == 0
    assert b"null" in buf.value
