"""MatrixMarket ingest (bmfp_mm_read_csr): the inverse of the reference's
write_mm (common/matrix_converters.h:119-144), then CSR -> BCSR to reach the
kernels. Host code only: runs on CPU."""
import os

import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm
from conftest import GOLDEN


def test_reads_back_what_write_mm_wrote(lib):
    # The golden file is the reference's write_mm output for gen_n_diag_bcsr(6, 3, 2).
    rp, c, v, n_cols = bm.mm_read_csr(os.path.join(GOLDEN, "ndiag_6x3_bs2.mtx"))
    brp, bc, bv = bm.gen_n_diag_bcsr(6, 3, 2)
    crp, cc, cv = bm.bcsr_to_csr(brp, bc, bv, 2)
    assert n_cols == 12
    assert np.array_equal(rp, crp) and np.array_equal(c, cc)
    assert np.array_equal(v.view(np.uint64), cv.view(np.uint64))  # %10.20g round-trips doubles
    # and back to the blocks the kernels take
    rbrp, rbc, rbv = bm.csr_to_bcsr(rp, c, v, n_cols, 2)
    assert np.array_equal(rbrp, brp) and np.array_equal(rbc, bc)
    assert np.array_equal(rbv.view(np.uint64), bv.view(np.uint64))


def test_symmetric_pattern_duplicates_and_order(lib, tmp_path):
    f = tmp_path / "m.mtx"
    f.write_text("%%MatrixMarket matrix coordinate real symmetric\n% a comment\n\n"
                 "4 4 5\n3 1 2.5\n1 1 1\n4 4 -3\n3 1 0.5\n2 2 7e-1\n")
    rp, c, v, n = bm.mm_read_csr(f)
    dense = np.zeros((4, 4))
    for r in range(4):
        for e in range(rp[r], rp[r + 1]):
            dense[r, c[e]] = v[e]
    want = np.array([[1, 0, 3.0, 0], [0, 0.7, 0, 0], [3.0, 0, 0, 0], [0, 0, 0, -3]])
    assert np.array_equal(dense, want) and n == 4
    assert all(np.all(np.diff(c[rp[r]:rp[r + 1]]) > 0) for r in range(4))
    g = tmp_path / "p.mtx"
    g.write_text("%%MatrixMarket matrix coordinate pattern skew-symmetric\n3 3 1\n3 2\n")
    rp, c, v, _ = bm.mm_read_csr(g, np.float32)
    assert v.dtype == np.float32 and list(rp) == [0, 0, 1, 2] and list(c) == [2, 1] and list(v) == [-1.0, 1.0]


@pytest.mark.parametrize("text,status", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", bm.ERROR_NOT_SUPPORTED),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", bm.ERROR_NOT_SUPPORTED),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n", bm.ERROR_INVALID_VALUE),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n", bm.ERROR_INVALID_VALUE),
    ("not a banner\n", bm.ERROR_INVALID_VALUE),
])
def test_rejects_what_it_cannot_read(lib, tmp_path, text, status):
    f = tmp_path / "bad.mtx"
    f.write_text(text)
    with pytest.raises(bm.BmfpError) as e:
        bm.mm_read_csr(f)
    assert e.value.status == status


def test_missing_file(lib, tmp_path):
    with pytest.raises(bm.BmfpError):
        bm.mm_read_csr(tmp_path / "nope.mtx")
