"""A compiled C++ caller of the reference's interface (tests/cxx/dropin_caller.cpp): it includes
include/core.h and include/sptrsv_syncfree_opencl.h and links libsptrsv_gb300.so where a
reference build links lib_SPTRSV.  On the CPU the program must compile and link with every
solver symbol resolved by the library; on the GPU it must run and match its own serial solve."""
import os
import shutil
import subprocess

import pytest

from sptrsv_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "dropin_caller.cpp")
SYMBOLS = ["base_gauss_upper", "barrier_upper", "setLevelUpAndGetMaxLevel", "sptrsv_syncfree_opencl",
           "sptrsv_syncfree3_opencl"]


def _build(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    _lib.lib()  # fails loudly when the library is not built
    lib = _lib.LIB_PATH
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "dropin_caller")
    cmd = [gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), SRC, "-L" + libdir, "-lsptrsv_gb300",
           "-Wl,-rpath," + libdir, "-Wl,--no-undefined", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, lib


def test_cxx_caller_links_against_library(tmp_path):
    exe, lib = _build(tmp_path)
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("no nm")
    undef = subprocess.run([nm, "-C", "-u", exe], capture_output=True, text=True).stdout
    defined = subprocess.run([nm, "-C", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for name in SYMBOLS:
        assert name + "(" in undef, name      # the program calls it ...
        assert name + "(" in defined, name    # ... and the library defines it


@pytest.mark.gpu
def test_cxx_caller_runs_on_gpu(tmp_path):
    exe, _ = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "dropin_caller ok" in r.stdout
