"""CPU checks of the C ABI library: it loads and exports every symbol include/ptg.h
declares (no compute call is made without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ptg_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_all_declared_symbols(pkg):
    lib_path = pkg._lib.LIB_PATH
    if not os.path.exists(lib_path):
        pytest.fail("libptg.so is not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(lib_path)
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"
    assert set(pkg._lib.EXPORTS) <= declared


def test_version_and_error_without_gpu(pkg):
    lib = pkg._lib.load()
    assert lib.ptg_version().startswith(b"ptg")
    # an invalid call fails with a status code and a message, without touching a GPU
    rc = lib.ptg_tensor_norms(None, None, None)
    assert rc == pkg._lib.PTG_ERR_INVALID
    assert b"NULL" in lib.ptg_last_error()


def test_default_options_match_reference(pkg):
    o = pkg.Options(order=3).to_c()
    # include/PARTENSOR_basic.hpp:176-218
    assert o.threshold_error == 1e-3 and o.nesterov_delta_1 == 1e-2 and o.nesterov_delta_2 == 1e-2
    assert o.max_iter == 20 and o.accel_coeff == 3 and o.accel_fail == 0
    assert o.acceleration == 1 and o.normalization == 1
    assert list(o.constraints)[:3] == [1, 1, 1]
