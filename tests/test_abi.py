"""The C-ABI library builds, loads and exports every symbol of include/wf.h.

CPU-only: no compute call is made without a GPU.
"""
import ctypes as C
import os
import re
import subprocess

import pytest

from weldformfem_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"WF_API\s+[\w\s\*]+?\b(wf_\w+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    return B.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "wf_init" in names and "wf_run" in names and "wf_add_box_length" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(wf_\w+)", out))
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, missing
    # nothing but the C ABI is exported
    extra = [n for n in exported if n not in declared_symbols()]
    assert not extra, extra


def test_library_loads_and_reports(libpath):
    L = C.CDLL(libpath)
    L.wf_abi_version.restype = C.c_int32
    assert L.wf_abi_version() == 1
    L.wf_status_string.restype = C.c_char_p
    L.wf_status_string.argtypes = [C.c_int]
    assert L.wf_status_string(0) == b"ok"
    assert L.wf_status_string(3) == b"CUDA error"
    L.wf_last_error.restype = C.c_char_p
    L.wf_last_error.argtypes = [C.c_void_p]
    assert L.wf_last_error(None) == b"null domain"
    # null arguments are rejected before any CUDA call
    L.wf_domain_create.argtypes = [C.c_void_p]
    assert L.wf_domain_create(None) == 1
    L.wf_domain_destroy.argtypes = [C.c_void_p]
    assert L.wf_domain_destroy(None) == 1


def test_library_is_sm103a_only(libpath):
    src = open(os.path.join(ROOT, "weldformfem_gb300", "build.py")).read()
    assert "arch=compute_103a,code=sm_103a" in src
    assert src.count("-gencode") == 1
