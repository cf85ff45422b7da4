"""The C ABI library loads without a GPU and exports every entry point include/*.h declares."""
import ctypes
import os
import re
import subprocess

import pytest

import sptrsv_gb300
from sptrsv_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_c_names():
    src = open(os.path.join(ROOT, "include", "sptrsv_gb300.h")).read()
    return sorted(set(re.findall(r"SPTRSV_API\s+[\w\s\*]+?\b(sptrsv_\w+)\s*\(", src)))


def _declared_cpp_names():
    names = []
    for h in ("core.h", "sptrsv_syncfree_opencl.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        names += re.findall(r"SPTRSV_API\s+(?:double|int)\s+(\w+)\s*\(", src)
    return sorted(set(names))


def test_library_loads():
    L = _lib.lib()
    assert L is not None


def test_every_c_symbol_exported():
    L = _lib.lib()
    names = _declared_c_names()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.C_API, n


def test_every_reference_signature_exported():
    names = _declared_cpp_names()
    assert set(names) == set(_lib.DROPIN_SYMBOLS), names
    L = _lib.lib()
    for n in names:
        assert hasattr(L, _lib.DROPIN_SYMBOLS[n]), n
    out = subprocess.run(["nm", "-DC", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    for sig in ["base_gauss_upper(int, double*, unsigned long*, int*, double*, double*, int)",
                "setLevelUpAndGetMaxLevel(int, int*, unsigned long*, unsigned long*)",
                "sptrsv_syncfree_opencl(int*, int*, double*, int, int, int, double*, double*, int)",
                "ccs2ccs_pad(double*, int*, unsigned long*, double*, unsigned long*, int*, int*, int&, int&)"]:
        assert sig in out, sig


def test_status_strings_and_defaults():
    assert sptrsv_gb300.status_string(0) == "ok"
    assert "diagonal" in sptrsv_gb300.status_string(-5)
    o = sptrsv_gb300.make_opts()
    assert o.tol == 1e-12 and o.max_refine == 8 and o.spin_budget_ns == 2_000_000_000


def test_no_device_is_an_error_not_a_crash():
    from tests.conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = _lib.lib().sptrsv_create(ctypes.byref(h), 0)
    assert rc in (-12, -3)


def test_product_does_not_import_the_oracle():
    pkg = os.path.join(ROOT, "sptrsv_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.replace("oracle is", ""), f
