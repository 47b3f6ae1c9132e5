"""The Golden Gate truss generator (bmfp_gen_golden_gate_bridge) against the
reference's own output (tests/golden/bridge_f64.npz, made by
fem_2d/golden_gate_bridge.h compiled in place), its structure at the size
main.cpp:349-381 builds, and the reference's solve of it on the GPU."""
import numpy as np
import pytest
import scipy.sparse as sp

import block_matrix_format_performance_gb300 as bm
from conftest import load_golden


def test_bridge_is_bitwise_the_reference_output(lib):
    g = load_golden("bridge_f64.npz")
    rp, c, v, rhs = bm.gen_golden_gate_bridge(1280.0, 345.0, 230.0, 7.62, 450.0, -2e6)
    assert rp.size - 1 == int(g["n_block_rows"]) and c.size == int(g["nnzb"])
    for mine, ref in ((rp, g["bcsr_row_ptr"]), (c, g["bcsr_cols"]), (v, g["bcsr_vals"]), (rhs, g["rhs"])):
        assert mine.dtype == ref.dtype and np.array_equal(mine.view(np.uint8), np.ascontiguousarray(ref).view(np.uint8))
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    assert np.array_equal(crp, g["csr_row_ptr"]) and np.array_equal(cc, g["csr_cols"])
    assert np.array_equal(cv.view(np.uint64), g["csr_vals"].view(np.uint64))


def test_main_cpp_bridge_structure(lib):
    # main.cpp:352-365: a 128 km main span, 260 m towers
    rp, c, v, rhs = bm.gen_golden_gate_bridge(128000.0, 345.0, 260.0, 7.62, 450.0, -2e6)
    n = rp.size - 1
    assert n > 50000 and np.all(np.diff(rp) >= 1) and (c.size - n) % 2 == 0
    for i in range(0, n, 997):
        row = c[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) >= 0) and i in row
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    K = sp.csr_matrix((cv, cc, crp), shape=(2 * n, 2 * n))
    assert abs(K - K.T).max() <= 1e-9 * abs(K).max()  # element blocks are symmetric
    # supported DOFs stay zero rows (golden_gate_bridge.h:815-855): the two
    # deck ends and both tower feet
    zero_rows = np.nonzero(abs(K).sum(axis=1).A1 == 0)[0]
    assert len(zero_rows) == 2 * 6
    loaded = np.nonzero(rhs)[0]
    assert len(loaded) > 0 and np.all(loaded % 2 == 1) and np.all(rhs[loaded] == -2e6)


def test_float_bridge_has_the_same_pattern(lib):
    rp, c, v, rhs = bm.gen_golden_gate_bridge()
    rp32, c32, v32, rhs32 = bm.gen_golden_gate_bridge(dtype=np.float32)
    assert np.array_equal(rp, rp32) and np.array_equal(c, c32) and v32.dtype == np.float32
    # the float model computes its geometry in float (cable coefficients cancel
    # large squares), so entries agree to about 1e-5 of the largest
    scale = np.abs(v).max()
    assert np.max(np.abs(v32.astype(np.float64) - v)) <= 1e-4 * scale
    assert np.array_equal(rhs32.astype(np.float64), rhs)


@pytest.mark.parametrize("args", [(0.0, 345.0, 230.0, 7.62), (1280.0, 345.0, 230.0, 0.0),
                                  (1280.0, float("nan"), 230.0, 7.62), (1e12, 345.0, 230.0, 7.62)])
def test_invalid_bridges_are_refused(lib, args):
    with pytest.raises(bm.BmfpError):
        bm.gen_golden_gate_bridge(*args)


@pytest.mark.gpu
def test_bridge_solve_as_main_cpp_does(lib, orc, cuda):
    # main.cpp:373-374: Jacobi-preconditioned BiCGStab, epsilon 0.8 on the
    # recursive residual, 1000 iterations; the oracle restates that loop.
    rp, c, v, rhs = bm.gen_golden_gate_bridge()
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    s = bm.Solver(A, "fp64", tol=0.8, max_iters=1000, preconditioner="jacobi", check_true_residual=False)
    x, info = s.solve_host(rhs)
    s.close(), A.close()
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    xo, st, it_o, _ = orc.bicgstab(crp, cc, cv, rhs, 0.8, 1000, True)
    assert info["status"] == bm.SUCCESS and info["recursive_rel_residual"] < 0.8
    assert abs(info["iterations"] - it_o) <= 0.25 * it_o + 10, (info, it_o)
    # the reference's rule looks at the recursive residual only; the true one
    # is not evaluated in that mode (reported as NaN)
    assert np.isnan(info["true_rel_residual"])
    K = sp.csr_matrix((cv, cc, crp))
    rel = np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs)
    assert abs(rel - info["recursive_rel_residual"]) <= 1e-6 * rel


def test_bridge_geometry_matches_the_matrix(lib):
    # bmfp_golden_gate_bridge_geometry: the nodes and bars behind the matrix
    import ctypes
    L = bm.load()
    args = (bm.R64F, 1280.0, 345.0, 230.0, 7.62)
    seg, nn, ne = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert L.bmfp_golden_gate_bridge_geometry(*args, ctypes.byref(seg), ctypes.byref(nn), ctypes.byref(ne),
                                              None, None, None, None) == 0
    xs, ys = np.zeros(nn.value), np.zeros(nn.value)
    st, en = np.zeros(ne.value, np.int32), np.zeros(ne.value, np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert L.bmfp_golden_gate_bridge_geometry(*args, ctypes.byref(seg), ctypes.byref(nn), ctypes.byref(ne),
                                              p(xs), p(ys), p(st), p(en)) == 0
    rp, c, v, rhs = bm.gen_golden_gate_bridge()
    assert nn.value == rp.size - 1 and c.size == nn.value + 2 * ne.value
    assert np.all(st < en) and en.max() < nn.value
    # every bar is a pair of off-diagonal blocks in the pattern
    for a, b in zip(st[::37], en[::37]):
        assert b in c[rp[a]:rp[a + 1]] and a in c[rp[b]:rp[b + 1]]
    # deck nodes 4s, 4s+1 lie on the top chord (78 m), the towers reach 230 m
    assert np.all(ys[0:4 * seg.value:4] == 78.0) and ys.max() == 230.0
    # loads sit on top-chord nodes inside the window around mid-span
    loaded = np.nonzero(rhs)[0] // 2
    mid = (1280.0 + 2 * 345.0) / 2
    assert np.all(np.abs(xs[loaded] - mid) < 450.0) and np.all(loaded % 4 <= 1)
