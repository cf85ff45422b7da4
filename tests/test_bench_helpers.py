"""Host logic of bench.py that needs no GPU: the errors it reports against the serial FP64 solve."""
import numpy as np

import bench
from oracle import oracle
from sptrsv_gb300 import gen


def test_errors_vs_serial_reports_each_solution():
    m = gen.random_upper(2000, 8.0, 0.9, 64, 5)
    xs, b = gen.system(m, 6)
    exact = oracle.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, 1)
    out = bench.errors_vs_serial(m, b, {"same": exact, "perturbed": exact * (1.0 + 1e-9)})
    assert out["oracle"].startswith("serial base_gauss_upper")
    assert out["same"]["max_elem_rel_error"] == 0.0 and out["same"]["rel_residual"] <= 1e-15
    assert abs(out["perturbed"]["max_elem_rel_error"] - 1e-9) <= 1e-12
    assert 1e-10 <= out["perturbed"]["rel_residual"] <= 1e-8
    assert abs(out["perturbed"]["rel_error_2norm"] - 1e-9) <= 1e-12
