"""The CPU oracle pinned against golden vectors from the reference's own code.

Fixtures in tests/golden/ come from tests/golden/make_golden.py, which runs the
reference headers compiled in place (oracle/_ref). Conversions and generators
must match bit for bit.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_golden

NDIAG = golden_cases("ndiag_")


@pytest.mark.parametrize("name", NDIAG)
def test_gen_n_diag_matches_reference(orc, name):
    g = load_golden(name)
    dt = g["bcsr_vals"].dtype
    rp, c, v = orc.gen_n_diag_bcsr(int(g["n_block_rows"]), int(g["nnzb"]) // int(g["n_block_rows"]),
                                   int(g["bs"]), dt)
    assert np.array_equal(rp, g["bcsr_row_ptr"])
    assert np.array_equal(c, g["bcsr_cols"])
    assert np.array_equal(v.view(np.uint8), g["bcsr_vals"].view(np.uint8))


@pytest.mark.parametrize("name", NDIAG + ["bridge_f64.npz"])
def test_bcsr_to_csr_matches_reference(orc, name):
    g = load_golden(name)
    rp, c, v = orc.bcsr_to_csr(g["bcsr_row_ptr"], g["bcsr_cols"], g["bcsr_vals"], int(g["bs"]))
    assert np.array_equal(rp, g["csr_row_ptr"])
    assert np.array_equal(c, g["csr_cols"])
    assert np.array_equal(v.view(np.uint8), g["csr_vals"].view(np.uint8))


@pytest.mark.parametrize("name", NDIAG + ["bridge_f64.npz"])
def test_transpose_blocks_matches_reference(orc, name):
    g = load_golden(name)
    bs = int(g["bs"])
    t = orc.transpose_blocks(g["bcsr_row_ptr"], g["bcsr_vals"], bs)
    assert np.array_equal(t.view(np.uint8), g["bcsr_vals_colmajor"].view(np.uint8))
    back = orc.transpose_blocks(g["bcsr_row_ptr"], t, bs)
    assert np.array_equal(back.view(np.uint8), g["bcsr_vals"].view(np.uint8))


@pytest.mark.parametrize("name", NDIAG + ["bridge_f64.npz"])
def test_csr_to_bcsr_inverts_reference_conversion(orc, name):
    g = load_golden(name)
    bs = int(g["bs"])
    n_cols = int(g["n_block_cols"]) * bs
    brp, bc, bv = orc.csr_to_bcsr(g["csr_row_ptr"], g["csr_cols"], g["csr_vals"], n_cols, bs)
    assert np.array_equal(brp, g["bcsr_row_ptr"])
    assert np.array_equal(bc, g["bcsr_cols"])
    assert np.array_equal(bv.view(np.uint8), g["bcsr_vals"].view(np.uint8))


def test_compare_results_matches_reference(orc):
    cases = json.load(open(os.path.join(GOLDEN, "compare_results.json")))
    assert any(c["flagged"] for c in cases) and not all(c["flagged"] for c in cases)
    for c in cases:
        dt = np.float64 if c["dtype"] == "f64" else np.float32
        _, flagged = orc.compare_results(np.array(c["a"], dt), np.array(c["b"], dt))
        assert flagged == c["flagged"]


@pytest.mark.parametrize("name", NDIAG + ["bridge_f64.npz"])
def test_bcsr_and_csr_spmv_agree_bitwise(orc, name):
    g = load_golden(name)
    bs = int(g["bs"])
    dt = g["bcsr_vals"].dtype
    x = np.random.default_rng(1).uniform(-1, 1, int(g["n_block_cols"]) * bs).astype(dt)
    y1 = orc.csr_spmv(g["csr_row_ptr"], g["csr_cols"], g["csr_vals"], x)
    y2 = orc.bcsr_spmv(g["bcsr_row_ptr"], g["bcsr_cols"], g["bcsr_vals"], bs, x)
    y3 = orc.csr_spmv(g["csr_row_ptr"], g["csr_cols"], g["csr_vals"], x, threads=3)
    assert np.array_equal(y1.view(np.uint8), y2.view(np.uint8))
    assert np.array_equal(y1.view(np.uint8), y3.view(np.uint8))


def test_csr_spmv_known_answer(orc):
    # x == 1 (as main.cpp:27 sets it): y_row = sum of the row's values.
    g = load_golden("ndiag_f64_n50_b6_bs2.npz")
    x = np.ones(100)
    y = orc.csr_spmv(g["csr_row_ptr"], g["csr_cols"], g["csr_vals"], x)
    rp = g["csr_row_ptr"]
    expect = np.array([g["csr_vals"][rp[i]:rp[i + 1]].sum() for i in range(100)])
    assert np.allclose(y, expect, rtol=1e-15, atol=0)


def test_band_generator_restatement_properties(orc):
    rp, c, v = orc.gen_band_bcsr(500, 8, 64, 2, seed=3)
    assert rp[0] == 0 and np.all(np.diff(rp) == 8)
    for i in range(500):
        row = c[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) > 0)
        assert row.min() >= max(0, i - 64) and row.max() <= min(499, i + 64)
    assert v.min() >= -1.0 and v.max() < 1.0
    # narrow windows near nothing: W < k gives W blocks
    rp2, c2, _ = orc.gen_band_bcsr(5, 8, 1, 1, seed=0)
    assert list(np.diff(rp2)) == [2, 3, 3, 3, 2]


def test_q4_dense_restatement_is_symmetric_and_rigid(orc):
    K, f = orc.q4_elasticity_dense(5, 3)
    assert np.allclose(K, K.T, atol=1e-15)
    ke = orc.q4_element_stiffness()
    # Rigid translations and the infinitesimal rotation give zero force.
    xs = np.array([0, 1, 1, 0.0]); ys = np.array([0, 0, 1, 1.0])
    for u in (np.tile([1.0, 0.0], 4), np.tile([0.0, 1.0], 4), np.ravel(np.column_stack([-ys, xs]))):
        assert np.abs(ke @ u).max() < 1e-14
    assert f.sum() == -3.0


def test_oracle_bicgstab_solves_small_elasticity(orc):
    K, f = orc.q4_elasticity_dense(8, 4)
    import scipy.sparse as sp
    A = sp.csr_matrix(K)
    A.eliminate_zeros()
    for precond in (False, True):
        x, st, it, rr = orc.bicgstab(A.indptr, A.indices, A.data, f, 1e-10, 2000, precond)
        assert st == 0, (st, it, rr)
        true_rel = np.linalg.norm(f - K @ x) / np.linalg.norm(f)
        assert true_rel < 1e-9
        xd = np.linalg.solve(K, f)
        assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-6
