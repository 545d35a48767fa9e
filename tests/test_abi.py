"""CPU-side checks of the C-ABI boundary: the library loads (no GPU needed to
dlopen it) and exports every entry point include/xflow.h declares."""
import ctypes as C
import os
import re

import pytest

from xflow_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "xflow.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(xf_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_match_binding():
    assert header_functions() == sorted(capi.EXPORTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(capi.LIB_PATH):
        pytest.fail("libxflow.so is not built (python -m xflow_gb300.build)")
    lib = C.CDLL(capi.LIB_PATH)
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_status_strings_without_gpu():
    L = capi.lib()
    assert L.xf_status_string(capi.XF_ERR_MASK).decode()
    assert L.xf_status_string(capi.XF_MAXIT).decode() == "iteration cap reached"
