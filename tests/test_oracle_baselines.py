"""The oracle's C generator and threaded BiCGStab — the inputs and the timed
loop of the CPU baselines (bench.py's cpu_baseline, cpu_solve and the
reference arm) — pinned to the numpy restatement, to the product's generator
and to the single-thread oracle solve. CPU only."""
import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm


@pytest.mark.parametrize("bs", [1, 2, 3, 8, 32])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_c_band_generator_matches_numpy_and_product(lib, orc, bs, dtype):
    nbr = 260 if bs < 32 else 40
    ref = orc.gen_band_bcsr(nbr, 8, 16, bs, 7, dtype)
    got = orc.gen_band_c(nbr, 8, 16, bs, 7, dtype, threads=3)
    prod = bm.gen_band_bcsr(nbr, 8, 16, bs, 7, dtype)
    for a, b, c in zip(ref, got, prod):
        assert np.array_equal(a, b) and np.array_equal(b, c)
    csr = orc.gen_band_c(nbr, 8, 16, bs, 7, dtype, csr=True, threads=2)
    for a, b in zip(orc.bcsr_to_csr(*ref, bs), csr):
        assert np.array_equal(a, b)


def test_c_uniform_vector_matches_numpy(orc):
    for stream in (0, 2, 5):
        a = orc.gen_uniform_vector(5000, 3, stream)
        assert np.array_equal(a, orc.gen_uniform_vector_c(5000, 3, stream))
        assert np.array_equal(a.astype(np.float32), orc.gen_uniform_vector_c(5000, 3, stream, np.float32))


def test_threaded_bicgstab_reproduces_the_single_thread_oracle(lib, orc):
    rp, c, v, rhs = bm.gen_q4_elasticity(60, 15)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    x1, st1, it1, r1 = orc.bicgstab(crp, cc, cv, rhs, 1e-10, 20000)
    xm, stm, itm, rm = orc.bicgstab_mt(crp, cc, cv, rhs, 1e-10, 20000, 1)
    assert (st1, it1) == (stm, itm) and r1 == rm
    assert np.array_equal(x1, xm)
    # several threads: another summation order, the same solve
    x4, st4, it4, r4 = orc.bicgstab_mt(crp, cc, cv, rhs, 1e-10, 20000, 4)
    assert st4 == 0 and r4 < 1e-10
    assert abs(it4 - it1) <= 0.25 * it1 + 10
    for pre in (False, True):
        xa, sa, ia, ra = orc.bicgstab(crp, cc, cv, rhs, 1e-10, 20000, pre)
        xb, sb, ib, rb = orc.bicgstab_mt(crp, cc, cv, rhs, 1e-10, 20000, 1, pre)
        assert ia == ib and np.array_equal(xa, xb)


def test_csr_spmv_into_a_given_buffer(orc):
    rp, c, v = orc.gen_band_c(300, 8, 16, 2, 1, csr=True)
    x = orc.gen_uniform_vector_c(600, 1, 2)
    y = np.full(600, np.nan)
    for th in (1, 3):
        orc.csr_spmv(rp, c, v, x, threads=th, out=y)
        assert np.array_equal(y, orc.csr_spmv(rp, c, v, x))


def test_oracle_block_jacobi_inverse_and_solve(lib, orc):
    rp, c, v, rhs = bm.gen_q4_elasticity(40, 10)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    M = orc.block_jacobi(crp, cc, cv, 2)
    D = v.reshape(-1, 2, 2)[np.repeat(np.arange(400), np.diff(rp)) == c]
    inv = np.linalg.inv(D)
    assert np.max(np.abs(M - inv)) <= 1e-14 * np.abs(inv).max()
    x, st, it, rel = orc.bicgstab_block_jacobi(crp, cc, cv, 2, rhs, 1e-10, 20000)
    y = orc.csr_spmv(crp, cc, cv, x)
    assert st == 0 and rel < 1e-10 and np.linalg.norm(rhs - y) / np.linalg.norm(rhs) < 1e-9
    # a zero diagonal block becomes the identity
    v0 = v.copy().reshape(-1, 2, 2)
    k = int(np.where((np.repeat(np.arange(400), np.diff(rp)) == c))[0][5])
    v0[k] = 0.0
    crp0, cc0, cv0 = orc.bcsr_to_csr(rp, c, v0.reshape(-1), 2)
    assert np.array_equal(orc.block_jacobi(crp0, cc0, cv0, 2)[5], np.eye(2))
