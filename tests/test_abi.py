"""The C-ABI library loads without a GPU and exports every function that
include/zpic_cuda.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(zc1?_[a-z_0-9]+)\s*\(", text)) - {"zc_inject_fn"})


@pytest.fixture(scope="module")
def lib():
    from zpic_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = declared("zpic_cuda.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from zpic_gb300 import _zc

    assert sorted(_zc.EXPORTS) == declared("zpic_cuda.h")


def test_status_strings(lib):
    lib.zc_status_string.restype = ctypes.c_char_p
    assert lib.zc_status_string(0) == b"ok"
    assert lib.zc_status_string(4) == b"particle escaped its cell"
    lib.zc_phase_name.restype = ctypes.c_char_p
    assert lib.zc_phase_name(0) == b"push"
