"""The C-ABI library builds for sm_103a, loads, and exports every function
include/stile_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

from stile_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "stile_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|int32_t)\s+(stile_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["stile_spmm_plan_upload", "stile_spmm_run", "stile_sddmm_run", "stile_csr_spmm_run",
              "stile_spmm_dvals", "stile_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    path = _lib.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes table covers the header
    assert set(declared_functions()) <= set(_lib.EXPORTS)


def test_invalid_arguments_are_reported_not_aborted():
    lib = _lib.load()
    h = _lib.SpmmPlanHost()
    h.M, h.K, h.tc_n_items = 4, 4, -1
    out = ctypes.c_void_p()
    rc = lib.stile_spmm_plan_upload(ctypes.byref(h), ctypes.byref(out))
    assert rc == -1
    assert "negative" in _lib.last_error()
    assert lib.stile_spmm_run(None, None, 0, None, 0, 4, None) == -1
    assert lib.stile_csr_spmm_run(-1, 0, None, None, None, None, None, 4, None, 4, 4, None) == -1
