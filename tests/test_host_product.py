"""Host-side product code (libbmfp.so, no GPU) against the golden vectors and
the oracle: conversions and generators must match bit for bit."""
import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm
from conftest import golden_cases, load_golden

NDIAG = golden_cases("ndiag_")


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("name", NDIAG)
def test_product_gen_n_diag_matches_reference(lib, name):
    g = load_golden(name)
    nbr = int(g["n_block_rows"])
    rp, c, v = bm.gen_n_diag_bcsr(nbr, int(g["nnzb"]) // nbr, int(g["bs"]), g["bcsr_vals"].dtype)
    assert same_bits(rp, g["bcsr_row_ptr"]) and same_bits(c, g["bcsr_cols"])
    assert same_bits(v, g["bcsr_vals"])


@pytest.mark.parametrize("name", NDIAG + ["bridge_f64.npz"])
def test_product_conversions_match_reference(lib, name):
    g = load_golden(name)
    bs = int(g["bs"])
    rp, c, v = bm.bcsr_to_csr(g["bcsr_row_ptr"], g["bcsr_cols"], g["bcsr_vals"], bs)
    assert same_bits(rp, g["csr_row_ptr"]) and same_bits(c, g["csr_cols"]) and same_bits(v, g["csr_vals"])
    t = bm.transpose_blocks(g["bcsr_row_ptr"], g["bcsr_vals"], bs)
    assert same_bits(t, g["bcsr_vals_colmajor"])
    assert same_bits(bm.transpose_blocks(g["bcsr_row_ptr"], t, bs), g["bcsr_vals"])
    brp, bc, bv = bm.csr_to_bcsr(g["csr_row_ptr"], g["csr_cols"], g["csr_vals"],
                                 int(g["n_block_cols"]) * bs, bs)
    assert same_bits(brp, g["bcsr_row_ptr"]) and same_bits(bc, g["bcsr_cols"]) and same_bits(bv, g["bcsr_vals"])


def test_csr_to_bcsr_matches_oracle_on_ragged_input(lib, orc):
    # An arbitrary sparse CSR (not produced by the BCSR converter): empty rows,
    # partially filled blocks, unsorted columns inside a row.
    rng = np.random.default_rng(5)
    n, bs = 60, 3
    rows = []
    for i in range(n):
        k = 0 if i % 7 == 0 else rng.integers(1, 9)
        cols = rng.choice(n, size=k, replace=False)
        rows.append(cols)
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    c = np.concatenate(rows).astype(np.int32)
    v = rng.uniform(-1, 1, c.size)
    a = bm.csr_to_bcsr(rp, c, v, n, bs)
    b = orc.csr_to_bcsr(rp, c, v, n, bs)
    for u, w in zip(a, b):
        assert same_bits(u, w)
    # Round trip through BCSR -> CSR reproduces every stored entry.
    crp, cc, cv = bm.bcsr_to_csr(*a, bs)
    dense1 = np.zeros((n, n)); dense2 = np.zeros((n, n))
    for i in range(n):
        dense1[i, c[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        dense2[i, cc[crp[i]:crp[i + 1]]] = cv[crp[i]:crp[i + 1]]
    assert np.array_equal(dense1, dense2)


def test_csr_to_bcsr_rejects_bad_shapes(lib):
    with pytest.raises(bm.BmfpError):
        bm.csr_to_bcsr(np.array([0, 1, 2]), np.array([0, 1]), np.ones(2), 2, 3)


@pytest.mark.parametrize("bs,dtype", [(1, np.float64), (2, np.float64), (4, np.float32), (3, np.float64)])
def test_band_generator_matches_restated_spec(lib, orc, bs, dtype):
    a = bm.gen_band_bcsr(700, 8, 64, bs, seed=11, dtype=dtype)
    b = orc.gen_band_bcsr(700, 8, 64, bs, seed=11, dtype=dtype)
    for u, w in zip(a, b):
        assert same_bits(u, w)


def test_band_generator_edge_windows(lib, orc):
    for nbr, k, h in ((1, 8, 64), (5, 8, 1), (130, 8, 64), (20, 3, 0)):
        a = bm.gen_band_bcsr(nbr, k, h, 2, seed=9)
        b = orc.gen_band_bcsr(nbr, k, h, 2, seed=9)
        for u, w in zip(a, b):
            assert same_bits(u, w)


def test_uniform_vector_matches_restated_spec(lib, orc):
    for dt in (np.float64, np.float32):
        assert same_bits(bm.gen_uniform_vector(1000, 0, 2, dt), orc.gen_uniform_vector(1000, 0, 2, dt))


@pytest.mark.parametrize("nx,ny", [(2, 2), (5, 3), (9, 4)])
def test_q4_generator_matches_dense_restatement(lib, orc, nx, ny):
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    K, f = orc.q4_elasticity_dense(nx, ny)
    n = 2 * nx * ny
    D = np.zeros((n, n))
    for br in range(nx * ny):
        for e in range(rp[br], rp[br + 1]):
            D[2 * br:2 * br + 2, 2 * c[e]:2 * c[e] + 2] = v[4 * e:4 * e + 4].reshape(2, 2)
    assert np.abs(D - K).max() <= 1e-14 * np.abs(K).max()
    assert np.array_equal(rhs, f)
    # full 9-point stencil kept in the pattern: nnzb = (3nx-2)(3ny-2)
    assert rp[-1] == (3 * nx - 2) * (3 * ny - 2)


def test_q4_config_sizes(lib):
    rp, _, _, _ = bm.gen_q4_elasticity(200, 50)
    assert rp[-1] == 88504  # 200x50 nodes -> 20 000 DOFs


def test_q4_float32_is_rounded_float64(lib):
    _, _, v64, r64 = bm.gen_q4_elasticity(6, 4, np.float64)
    _, _, v32, r32 = bm.gen_q4_elasticity(6, 4, np.float32)
    assert same_bits(v64.astype(np.float32), v32) and same_bits(r64.astype(np.float32), r32)


def test_spmv_bytes_formula(lib):
    # values + block cols + row offsets + x once + y once
    nbr, bs, nnzb = 100_000, 4, 800_000
    assert bm.bcsr_spmv_bytes(np.float64, nbr, nbr, bs, nnzb) == nnzb * 16 * 8 + nnzb * 4 + (nbr + 1) * 4 + 2 * nbr * bs * 8
    assert bm.csr_spmv_bytes(np.float32, 10, 10, 30) == 30 * 4 + 30 * 4 + 11 * 4 + 2 * 10 * 4
