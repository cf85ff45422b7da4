"""The reference's file formats (utils.cpp:9-109) through the library's readers and writers:
round trips of the golden matrices, the text layout cross-read by the oracle's own reader, and the
MatrixMarket reading rule (a lower factor in column order read as the CSR of its transpose)."""
import numpy as np
import pytest

import sptrsv_gb300 as sp


@pytest.mark.parametrize("tag", ["csr_6_upper", "rand3000", "snr800"])
@pytest.mark.parametrize("ext", ["matrix", "txt"])
def test_csr_round_trip(golden, orc, tmp_path, tag, ext):
    rp, col, val = golden[tag + "/row_ptr"], golden[tag + "/col"], golden[tag + "/val"]
    path = tmp_path / f"m.{ext}"
    sp.write_csr(path, rp, col, val)
    rp2, col2, val2 = sp.read_csr(path)
    assert np.array_equal(rp2, rp) and np.array_equal(col2, col) and np.array_equal(val2, val)
    if ext == "txt":
        rp3, col3, val3 = orc.read_txt_csr(str(path))
        assert np.array_equal(rp3.astype(np.int64), rp) and np.array_equal(col3, col) and np.array_equal(val3, val)


def test_matrix_binary_layout(tmp_path):
    """int32 n, uint64 nz, int32 col[nz], uint64 row_ptr[n+1], f64 val[nz] (utils.cpp:17-31)."""
    rp = np.array([0, 2, 3], dtype=np.int64)
    col = np.array([0, 1, 1], dtype=np.int32)
    val = np.array([2.0, -1.0, 4.0])
    path = tmp_path / "t.matrix"
    sp.write_csr(path, rp, col, val)
    raw = path.read_bytes()
    expect = (np.int32(2).tobytes() + np.uint64(3).tobytes() + col.tobytes() + rp.astype(np.uint64).tobytes()
              + val.tobytes())
    assert raw == expect


@pytest.mark.parametrize("ext", ["snodes", "txt"])
def test_snodes_round_trip(golden, tmp_path, ext):
    sn = golden["snr800/snodes"].astype(np.int32)
    path = tmp_path / f"s.{ext}"
    sp.write_snodes(path, sn)
    assert np.array_equal(sp.read_snodes(path), sn)


def test_mtx_reads_lower_factor_as_transpose(golden, tmp_path):
    rp, col, val = golden["rand3000/row_ptr"], golden["rand3000/col"], golden["rand3000/val"]
    n = len(rp) - 1
    # U^T written as MatrixMarket coordinates in column order (column j of U^T = row j of U)
    lines = ["%%MatrixMarket matrix coordinate real general", "% lower factor", f"{n} {n} {len(col)}"]
    for j in range(n):
        for k in range(rp[j], rp[j + 1]):
            lines.append(f"{col[k] + 1} {j + 1} {float(val[k])!r}")
    path = tmp_path / "l.mtx"
    path.write_text("\n".join(lines) + "\n")
    rp2, col2, val2 = sp.read_csr(path)
    assert np.array_equal(rp2, rp) and np.array_equal(col2, col) and np.array_equal(val2, val)


def test_errors(tmp_path):
    with pytest.raises(sp.SptrsvError) as e:
        sp.read_csr(tmp_path / "missing.matrix")
    assert e.value.status == -16
    with pytest.raises(sp.SptrsvError) as e:
        sp.read_csr(tmp_path / "m.unknown")
    assert e.value.status == -2
    (tmp_path / "short.matrix").write_bytes(np.int32(5).tobytes() + np.uint64(9).tobytes())
    with pytest.raises(sp.SptrsvError) as e:
        sp.read_csr(tmp_path / "short.matrix")
    assert e.value.status == -16
