"""The command-line front end with the reference's arguments (app/main.cpp:4-66): usage, unknown
algorithms, and every algorithm name on a matrix and partition written in the reference's file
formats, each result checked by the front end's own residual report."""
import re

import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300.__main__ import main


def test_usage_without_arguments(capsys):
    assert main([]) == 1
    assert "ALGO MATRIX SNODES NTHREADS NRHS OPT" in capsys.readouterr().out


def test_unknown_algorithm(golden, tmp_path, capsys):
    path = tmp_path / "m.matrix"
    sp.write_csr(path, golden["csr_6_upper/row_ptr"], golden["csr_6_upper/col"], golden["csr_6_upper/val"])
    assert main(["nope", str(path), str(path), "1", "1", "opt_false"]) == 1
    assert "Unknown algorithm nope" in capsys.readouterr().out


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ["base", "custom", "blas", "barrier", "syncfree", "write_first", "mkl"])
@pytest.mark.parametrize("opt", ["opt_false", "opt_true"])
def test_every_algorithm(golden, tmp_path, capsys, algo, opt):
    mpath, spath = tmp_path / "m.matrix", tmp_path / "m.snodes"
    sp.write_csr(mpath, golden["snr800/row_ptr"], golden["snr800/col"], golden["snr800/val"])
    sp.write_snodes(spath, golden["snr800/snodes"].astype(np.int32))
    assert main([algo, str(mpath), str(spath), "4", "3", opt, "check"]) == 0
    out = capsys.readouterr().out
    found = re.search(r"relative residual ([0-9.e+-]+); difference from the FP64 sync-free solve ([0-9.e+-]+)", out)
    assert found, out
    assert float(found.group(1)) <= 1e-12 and float(found.group(2)) <= 1e-12, out
