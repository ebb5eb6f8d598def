"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/pdgpu.h declares."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pdgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pdgpu_[a-z_0-9]+)\s*\(", txt)))


def test_library_builds_and_exports_every_declared_symbol():
    from pd_gb300 import build, ffi
    path = build.build()
    L = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 18
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(syms) == set(ffi.SIGNATURES)


def test_error_strings_without_gpu():
    from pd_gb300 import ffi
    L = ffi.load()
    assert L.pdgpu_error_string(0) == b"ok"
    assert b"NaN" in L.pdgpu_error_string(-5)


def test_create_rejects_bad_description_without_touching_a_gpu():
    from pd_gb300 import ffi
    L = ffi.load()
    st = ctypes.c_int(0)
    assert not L.pdgpu_create(0, None, ctypes.byref(st))
    assert st.value == -1
