"""BiCGStab on the GPU against the oracle's restatement of the reference loop
(gpu/bicgstab.cu:387-513) and an independent FP64 direct solve.

Bars: true relative residual ||b - A x|| / ||b|| below the tolerance, error
against the direct solve reported and bounded, iteration counts of the plain
recurrences (the oracle's algorithm) within 25 % (+10) of the oracle's (the
dot products sum in a different order; BiCGStab's erratic residual history on
these operators turns that into a different iteration count, most visibly
with Jacobi), and bitwise repeatability.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

import block_matrix_format_performance_gb300 as bm

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bcsr_dense_csr(rp, c, v, bs):
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, bs)
    n = (len(rp) - 1) * bs
    return sp.csr_matrix((cv, cc, crp), shape=(n, n))


def diag_dominant_bcsr(nbr, bs, seed, extra=8):
    """Random BCSR with a dominant diagonal block in every block row."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(nbr):
        cand = np.unique(np.concatenate([[i], rng.integers(max(0, i - 20), min(nbr, i + 21), extra)]))
        rows.append(cand)
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    c = np.concatenate(rows).astype(np.int32)
    v = rng.uniform(-1, 1, c.size * bs * bs)
    for i in range(nbr):
        k = rp[i] + int(np.where(rows[i] == i)[0][0])
        blk = v[k * bs * bs:(k + 1) * bs * bs].reshape(bs, bs)
        blk += np.eye(bs) * (len(rows[i]) * bs * 1.5)
    return rp, c, v


@pytest.mark.parametrize("precond", ["none", "jacobi"])
@pytest.mark.parametrize("grid", [(24, 6), (50, 13), (100, 25)])
def test_fp64_q4_elasticity_matches_oracle(lib, orc, cuda, grid, precond):
    nx, ny = grid
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    s = bm.Solver(A, "fp64", tol=1e-10, max_iters=50000, preconditioner=precond)
    x, info = s.solve_host(rhs)
    K = bcsr_dense_csr(rp, c, v, 2)
    rel = np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs)
    assert info["status"] == bm.SUCCESS, info
    assert rel < 1e-10 and abs(rel - info["true_rel_residual"]) <= 1e-12 + 1e-3 * rel
    xd = sla.spsolve(K.tocsc(), rhs)
    err = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    assert err < 1e-5, err  # reported: forward error bounded by cond(A) * residual
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    xo, st, it_o, _ = orc.bicgstab(crp, cc, cv, rhs, 1e-10, 50000, precond == "jacobi")
    # Iteration counts compare the oracle's own algorithm: the plain
    # recurrences stopped on the recursive residual (no replacement, no
    # restart); the dot products still sum in another order.
    _, plain = bm.Solver(A, "fp64", tol=1e-10, max_iters=50000, preconditioner=precond,
                         check_true_residual=False).solve_host(rhs)
    assert plain["replacements"] == 0 and plain["restarts"] == 0
    assert abs(plain["iterations"] - it_o) <= 0.25 * it_o + 10, (plain, it_o, info)
    s.close(), A.close()


def test_recursive_only_mode_follows_reference_stop_rule(lib, orc, cuda):
    # check_true_residual = 0: stop when ||r_i|| / ||b|| < eps (gpu/bicgstab.cu:512)
    rp, c, v, rhs = bm.gen_q4_elasticity(40, 10)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    s = bm.Solver(A, "fp64", tol=1e-8, max_iters=10000, check_true_residual=False)
    x, info = s.solve_host(rhs)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    _, st, it_o, rr_o = orc.bicgstab(crp, cc, cv, rhs, 1e-8, 10000, False)
    assert info["status"] == bm.SUCCESS and info["recursive_rel_residual"] < 1e-8
    assert abs(info["iterations"] - it_o) <= 0.25 * it_o + 10
    assert info["restarts"] == 0


def test_solve_is_bitwise_repeatable(lib, cuda):
    rp, c, v, rhs = bm.gen_q4_elasticity(60, 15)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    s = bm.Solver(A, "fp64")
    x1, i1 = s.solve_host(rhs)
    x2, i2 = s.solve_host(rhs)
    assert i1["iterations"] == i2["iterations"]
    assert np.array_equal(x1.view(np.uint64), x2.view(np.uint64))


@pytest.mark.parametrize("bs", [1, 2, 3, 4, 8])
def test_fp64_diag_dominant_any_block_size(lib, cuda, bs):
    rp, c, v = diag_dominant_bcsr(300, bs, seed=bs)
    K = bcsr_dense_csr(rp, c, v, bs)
    b = np.random.default_rng(1).uniform(-1, 1, 300 * bs)
    A = bm.Matrix.from_bcsr(rp, c, v, bs)
    x, info = bm.Solver(A, "fp64").solve_host(b)
    assert info["status"] == bm.SUCCESS
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) < 1e-10
    xd = sla.spsolve(K.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9


def test_csr_matrix_solve_like_the_reference(lib, orc, cuda):
    """The reference solves CSR (csr_matrix_class); bs = 0 handles go through
    the CSR phase kernels."""
    rp, c, v, rhs = bm.gen_q4_elasticity(30, 8)
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    A = bm.Matrix.from_csr(crp, cc, cv, len(crp) - 1)
    for pre in ("none", "jacobi"):
        x, info = bm.Solver(A, "fp64", preconditioner=pre).solve_host(rhs)
        K = sp.csr_matrix((cv, cc, crp))
        assert info["status"] == bm.SUCCESS
        assert np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs) < 1e-10


def test_fp32_solver_reaches_fp32_tolerance(lib, cuda):
    rp, c, v = diag_dominant_bcsr(500, 2, seed=9)
    K = bcsr_dense_csr(rp, c, v, 2)
    b = np.random.default_rng(2).uniform(-1, 1, 1000)
    A32 = bm.Matrix.from_bcsr(rp, c, v.astype(np.float32), 2)
    x, info = bm.Solver(A32, "fp32", tol=1e-5).solve_host(b.astype(np.float32))
    assert info["status"] == bm.SUCCESS and info["iterations_fp32"] == info["iterations"]
    assert np.linalg.norm(b - K @ x.astype(np.float64)) / np.linalg.norm(b) < 1e-4


def test_mixed_precision_refines_to_fp64_accuracy(lib, cuda):
    rp, c, v = diag_dominant_bcsr(2000, 2, seed=4)
    K = bcsr_dense_csr(rp, c, v, 2)
    b = np.random.default_rng(3).uniform(-1, 1, 4000)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "mixed", tol=1e-10).solve_host(b)
    assert info["status"] == bm.SUCCESS, info
    assert info["used_fp64_fallback"] == 0 and info["iterations_fp32"] == info["iterations"]
    assert info["refinements"] >= 2
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) < 1e-10
    x64, i64 = bm.Solver(A, "fp64", tol=1e-10).solve_host(b)
    assert np.linalg.norm(x - x64) / np.linalg.norm(x64) < 1e-9


def test_mixed_precision_ill_conditioned_falls_back_and_converges(lib, cuda):
    """cond(A) ~ 1e6 for a 100x25 Q4 grid: FP32 inner solves stall; the solver
    finishes in FP64 and still meets the tolerance."""
    rp, c, v, rhs = bm.gen_q4_elasticity(100, 25)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "mixed", tol=1e-10, max_iters=50000).solve_host(rhs)
    K = bcsr_dense_csr(rp, c, v, 2)
    assert info["status"] == bm.SUCCESS, info
    assert np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reused_solver_gives_the_same_answer_every_time(lib, cuda, precision):
    """A solver object serves many right-hand sides (the server's whole-GPU
    lanes keep one per matrix): nothing of an earlier solve may leak into the
    next. Mixed precision on this grid runs FP64 only (the creation probe
    finds FP32 steps unable to progress on it), which once kept counting
    iterations across solves until the limit stopped it at x = 0."""
    rp, c, v, rhs = bm.gen_q4_elasticity(100, 25)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    K = bcsr_dense_csr(rp, c, v, 2)
    s = bm.Solver(A, precision, tol=1e-10, max_iters=3000)
    rng = np.random.default_rng(5)
    bs = [rhs, rng.uniform(-1, 1, rhs.size), rhs, rhs]
    out = [s.solve_host(b) for b in bs]
    for (x, info), b in zip(out, bs):
        assert info["status"] == bm.SUCCESS, info
        assert info["iterations"] <= 3000
        assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) < 1e-10
    # The same right-hand side gives the same bits whatever came before.
    for k in (2, 3):
        assert np.array_equal(out[0][0].view(np.uint64), out[k][0].view(np.uint64))
        assert out[0][1]["iterations"] == out[k][1]["iterations"]
    if precision == "mixed":
        # decided once per matrix: FP64 only from the first solve on, and then
        # bit for bit the FP64 solver's answer
        for _, info in out:
            assert info["iterations_fp32"] == 0 and info["used_fp64_fallback"] == 1
        x64, _ = bm.Solver(A, "fp64", tol=1e-10, max_iters=3000).solve_host(rhs)
        assert np.array_equal(out[0][0].view(np.uint64), x64.view(np.uint64))


@pytest.mark.parametrize("grid", [(97, 24), (150, 38), (240, 60)])
def test_fp64_reaches_the_tolerance_where_fp64_allows(lib, cuda, grid):
    """Grids of the uneven batch whose FP64 rounding floor u ||A| |x|| / ||b||
    lies below 1e-10 (1.7e-11, 3.1e-11 and 6.4e-11): the residual replacement
    keeps BiCGStab's recursive residual on the true one, so the solve ends
    below 1e-10 in b - A x (plain restarts from the true residual left these
    at 1.0-1.04e-10)."""
    nx, ny = grid
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64", tol=1e-10, max_iters=50000).solve_host(rhs)
    K = bcsr_dense_csr(rp, c, v, 2)
    rel = np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs)
    assert info["status"] == bm.SUCCESS and info["true_rel_residual"] < 1e-10, info
    assert rel < 1e-10, rel
    assert info["replacements"] >= 1, info
    floor = 2.0 ** -53 * np.linalg.norm(abs(K) @ abs(x)) / np.linalg.norm(rhs)
    assert floor < 1e-10


def test_replacement_off_keeps_the_plain_recurrences(lib, cuda):
    """residual_replacement = 0 runs the unmodified recurrences (no
    replacement happens); the restarts from the true residual remain."""
    rp, c, v, rhs = bm.gen_q4_elasticity(60, 15)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64", tol=1e-10, residual_replacement=0).solve_host(rhs)
    assert info["replacements"] == 0
    x1, info1 = bm.Solver(A, "fp64", tol=1e-10).solve_host(rhs)
    assert info1["replacements"] >= 1 and info1["status"] == bm.SUCCESS, info1


def test_zero_rhs_and_iteration_limit(lib, cuda):
    rp, c, v, rhs = bm.gen_q4_elasticity(30, 8)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64").solve_host(np.zeros_like(rhs))
    assert info["status"] == bm.SUCCESS and info["iterations"] == 0 and not x.any()
    x, info = bm.Solver(A, "fp64", max_iters=5).solve_host(rhs)
    assert info["status"] == bm.ERROR_NOT_CONVERGED and info["iterations"] == 5
    assert np.isfinite(x).all() and x.any()


def test_solver_rejects_bad_configurations(lib, cuda):
    rp, c, v = bm.gen_band_bcsr(10, 3, 2, 2, seed=0)
    A32 = bm.Matrix.from_bcsr(rp, c, v.astype(np.float32), 2)
    with pytest.raises(bm.BmfpError):
        bm.Solver(A32, "fp64")
    with pytest.raises(bm.BmfpError):
        bm.Solver(A32, "mixed")
    rect = bm.Matrix.from_bcsr(rp, c, v, 2, n_block_cols=12)
    with pytest.raises(bm.BmfpError):
        bm.Solver(rect, "fp64")


def test_mixed_finish_that_breaks_down_restarts_from_zero(lib, cuda):
    """Request 729 of the seeded serving stream (1000x250 elasticity grid,
    random load): FP64 BiCGStab started from the FP32-refined iterate breaks
    down again and again there, while plain FP64 from x = 0 converges. The
    mixed solver must then solve from x = 0 and reach plain FP64's result."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    _, grids = bench.serve_stream(1000, 2000.0)
    rng = np.random.default_rng(7)
    b = None
    for k, (nx, ny) in enumerate(grids[:730]):
        b = rng.uniform(-1, 1, 2 * nx * ny)
        b.reshape(ny, nx, 2)[:, 0, :] = 0.0
    assert grids[729] == (1000, 250)
    rp, c, v, _ = bm.gen_q4_elasticity(1000, 250)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x64, i64 = bm.Solver(A, "fp64", tol=1e-10).solve_host(b)
    xm, im = bm.Solver(A, "mixed", tol=1e-10).solve_host(b)
    assert i64["true_rel_residual"] < 1e-10
    assert im["used_fp64_fallback"] == 1
    assert im["true_rel_residual"] <= max(1e-10, 2 * i64["true_rel_residual"]), im


@pytest.mark.parametrize("grid", [(24, 6), (50, 13), (100, 25)])
def test_block_jacobi_q4_matches_oracle(lib, orc, cuda, grid):
    """Block-Jacobi right preconditioning (the inverse of each 2x2 diagonal
    block; the block form of gpu/bicgstab.cu:201-238) against the oracle's
    restatement. The default solve meets the tolerance in b - A x and the
    direct solve's answer. The plain recurrences (stop on the recursive
    residual, no replacement: the oracle's algorithm) reach the oracle's
    iteration count within 40 % (+10): the GPU sums its dot products in
    another order, and on these ill-conditioned operators BiCGStab's
    erratic residual history turns that into a different count (24x6:
    87 against 136 iterations with replacement on)."""
    nx, ny = grid
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64", tol=1e-10, max_iters=50000, preconditioner="block_jacobi").solve_host(rhs)
    K = bcsr_dense_csr(rp, c, v, 2)
    rel = np.linalg.norm(rhs - K @ x) / np.linalg.norm(rhs)
    assert info["status"] == bm.SUCCESS and rel < 1e-10, info
    xd = sla.spsolve(K.tocsc(), rhs)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-5
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    _, st, it_o, _ = orc.bicgstab_block_jacobi(crp, cc, cv, 2, rhs, 1e-10, 50000)
    assert st == 0
    _, plain = bm.Solver(A, "fp64", tol=1e-10, max_iters=50000, preconditioner="block_jacobi",
                         check_true_residual=False).solve_host(rhs)
    assert plain["replacements"] == 0 and plain["restarts"] == 0
    assert abs(plain["iterations"] - it_o) <= 0.4 * it_o + 10, (plain, it_o)
    A.close()


@pytest.mark.parametrize("bs", [3, 4, 8])
def test_block_jacobi_any_block_size(lib, orc, cuda, bs):
    """The generic block-row routine (bs 3-8): a matrix whose diagonal
    blocks dominate, where block Jacobi is close to exact: few iterations,
    fewer than without a preconditioner, and the oracle's count."""
    rp, c, v = diag_dominant_bcsr(400, bs, seed=20 + bs)
    K = bcsr_dense_csr(rp, c, v, bs)
    b = np.random.default_rng(bs).uniform(-1, 1, 400 * bs)
    A = bm.Matrix.from_bcsr(rp, c, v, bs)
    x, info = bm.Solver(A, "fp64", preconditioner="block_jacobi").solve_host(b)
    _, i0 = bm.Solver(A, "fp64").solve_host(b)
    assert info["status"] == bm.SUCCESS
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) < 1e-10
    assert info["iterations"] <= i0["iterations"]
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, bs)
    _, st, it_o, _ = orc.bicgstab_block_jacobi(crp, cc, cv, bs, b, 1e-10, 20000)
    assert st == 0 and abs(info["iterations"] - it_o) <= 0.25 * it_o + 10 + 50 * info["restarts"], (info, it_o)
    # FP32 values through the same routine
    A32 = bm.Matrix.from_bcsr(rp, c, v.astype(np.float32), bs)
    x32, i32 = bm.Solver(A32, "fp32", tol=1e-5, preconditioner="block_jacobi").solve_host(b.astype(np.float32))
    assert i32["status"] == bm.SUCCESS
    assert np.linalg.norm(b - K @ x32.astype(np.float64)) / np.linalg.norm(b) < 1e-4


def test_block_jacobi_of_bs1_is_point_jacobi(lib, cuda):
    """With 1x1 blocks the block inverse is 1/a_ii: the same solve, bit for
    bit, as point Jacobi."""
    rp, c, v, rhs = bm.gen_q4_elasticity(30, 8)
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    A = bm.Matrix.from_csr(crp, cc, cv, len(crp) - 1)
    xb, ib = bm.Solver(A, "fp64", preconditioner="block_jacobi").solve_host(rhs)
    xp, ip = bm.Solver(A, "fp64", preconditioner="jacobi").solve_host(rhs)
    assert ib["iterations"] == ip["iterations"]
    assert np.array_equal(xb.view(np.uint64), xp.view(np.uint64))


def test_block_jacobi_limits(lib, cuda):
    rp, c, v = bm.gen_band_bcsr(20, 3, 2, 16, seed=0)
    A = bm.Matrix.from_bcsr(rp, c, v, 16)
    with pytest.raises(bm.BmfpError) as e:
        bm.Solver(A, "fp64", preconditioner="block_jacobi")
    assert e.value.status == bm.ERROR_NOT_SUPPORTED
    rp, c, v, _ = bm.gen_q4_elasticity(20, 5)
    m = bm.Matrix.from_bcsr(rp, c, v, 2)
    with pytest.raises(bm.BmfpError):
        bm.Batch([m], "fp64", preconditioner=bm.PRECOND_BLOCK_JACOBI)


def test_breakdown_restart_takes_a_new_shadow_residual(lib, cuda):
    """Request 3331 of the 5000-request serving stream (1000x250 grid, random
    load) on the whole-GPU solver as the server's wide lanes run it (one CTA
    per SM): BiCGStab breaks down there, and restarts from the true residual
    with the same shadow vector (rh = r) broke down again, ending at 2.3e-6.
    A restart after a breakdown now takes a perturbed shadow residual."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    _, grids = bench.serve_stream(5000, 2000.0)
    rng = np.random.default_rng(7)
    b = None
    for nx, ny in grids[:3332]:
        b = rng.uniform(-1, 1, 2 * nx * ny)
        b.reshape(ny, nx, 2)[:, 0, :] = 0.0
    assert grids[3331] == (1000, 250)
    rp, c, v, _ = bm.gen_q4_elasticity(1000, 250)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64", tol=1e-10, ctas_per_sm=1).solve_host(b)
    K = bcsr_dense_csr(rp, c, v, 2)
    rel = np.linalg.norm(b - K @ x) / np.linalg.norm(b)
    floor = bench.fp64_floor(rp, c, v, 2, x, b)
    assert info["status"] != bm.ERROR_BREAKDOWN, info
    assert rel < max(1e-10, 2 * floor), (rel, floor, info)
    A.close()


def _solve_modes(A, b, precision, **kw):
    """The same solve with the graph of phase kernels and with the persistent
    iteration kernel."""
    out = []
    for mode in ("graph", "persistent"):
        s = bm.Solver(A, precision, launch_mode=mode, **kw)
        out.append(s.solve_host(b))
        s.close()
    return out


def _same_bits(a, b):
    return a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("case", ["q4", "q4_plain", "q4_jacobi", "q4_cps1", "q4_cps2", "csr", "bs3", "bs4", "bs5",
                                  "fp32", "fp32_jacobi", "mixed", "tiny"])
def test_persistent_iterations_give_the_graphs_bits(lib, cuda, case):
    """The persistent kernel runs the phase bodies between grid barriers and
    derives the scalars in every CTA from the same partials, in the same
    order, as the phase kernels' last CTA: the same bits, iterations,
    replacements and restarts, for every product kind it serves."""
    kw = {"ctas_per_sm": 3}  # the persistent kernel's most; the graph then runs the same grid
    precision = "fp64"
    if case.startswith("q4"):
        rp, c, v, b = bm.gen_q4_elasticity(100, 25)
        A = bm.Matrix.from_bcsr(rp, c, v, 2)
        if case == "q4_jacobi":
            kw["preconditioner"] = "jacobi"
        if case == "q4_plain":  # the reference's recurrences: no replacement, no true-residual restarts
            kw["check_true_residual"] = False
        if case == "q4_cps1":
            kw["ctas_per_sm"] = 1
        if case == "q4_cps2":
            kw["ctas_per_sm"] = 2
    elif case == "csr":
        rp, c, v, b = bm.gen_q4_elasticity(30, 8)
        crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
        A = bm.Matrix.from_csr(crp, cc, cv, len(crp) - 1)
        kw["preconditioner"] = "jacobi"
    elif case in ("bs3", "bs4", "bs5"):
        bs = int(case[2])
        rp, c, v = diag_dominant_bcsr(400, bs, seed=bs)
        b = np.random.default_rng(3).uniform(-1, 1, 400 * bs)
        A = bm.Matrix.from_bcsr(rp, c, v, bs)
    elif case in ("fp32", "fp32_jacobi"):
        rp, c, v = diag_dominant_bcsr(500, 2, seed=9)
        b = np.random.default_rng(2).uniform(-1, 1, 1000).astype(np.float32)
        A = bm.Matrix.from_bcsr(rp, c, v.astype(np.float32), 2)
        precision = "fp32"
        kw["tol"] = 1e-5
        if case == "fp32_jacobi":
            kw["preconditioner"] = "jacobi"
    elif case == "mixed":
        rp, c, v = diag_dominant_bcsr(500, 2, seed=9)
        b = np.random.default_rng(2).uniform(-1, 1, 1000)
        A = bm.Matrix.from_bcsr(rp, c, v, 2)
        precision = "mixed"
    else:  # a system smaller than one CTA: a grid of one
        rp, c, v = diag_dominant_bcsr(60, 2, seed=5)
        b = np.random.default_rng(4).uniform(-1, 1, 120)
        A = bm.Matrix.from_bcsr(rp, c, v, 2)
    (xg, ig), (xp, ip) = _solve_modes(A, b, precision, **kw)
    assert ip["status"] == bm.SUCCESS, ip
    for k in ("status", "iterations", "iterations_fp32", "refinements", "restarts", "replacements"):
        assert ig[k] == ip[k], (k, ig, ip)
    assert _same_bits(xg, xp)
    if case == "q4":
        assert ip["replacements"] >= 1  # the replacement iterations ran in the kernel too
    if case == "mixed":
        assert ip["iterations_fp32"] > 0  # and the FP32 engine's kernel
    A.close()


def test_persistent_launch_limits(lib, cuda):
    """Block Jacobi runs as graphs under auto and is refused when the
    persistent kernel is asked for. The persistent kernel runs at most 3
    CTAs per SM: asked for 8 on a system of 160 000 rows (625 CTAs) it runs
    the grid of 3, and gives the graph's bits at 3."""
    rp, c, v, b = bm.gen_q4_elasticity(24, 6)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    with pytest.raises(bm.BmfpError) as e:
        bm.Solver(A, "fp64", launch_mode="persistent", preconditioner="block_jacobi")
    assert e.value.status == bm.ERROR_NOT_SUPPORTED
    x, info = bm.Solver(A, "fp64", preconditioner="block_jacobi").solve_host(b)
    assert info["status"] == bm.SUCCESS
    rpl, cl, vl, bl = bm.gen_q4_elasticity(400, 200)
    AL = bm.Matrix.from_bcsr(rpl, cl, vl, 2)
    xp, ip = bm.Solver(AL, "fp64", launch_mode="persistent", ctas_per_sm=8, max_iters=200).solve_host(bl)
    xg, ig = bm.Solver(AL, "fp64", launch_mode="graph", ctas_per_sm=3, max_iters=200).solve_host(bl)
    assert ip["iterations"] == ig["iterations"] == 200
    assert _same_bits(xp, xg)
    with pytest.raises(bm.BmfpError) as e:
        bm.Solver(A, "fp64", launch_mode=3)
    assert e.value.status == bm.ERROR_INVALID_VALUE
    rp8, c8, v8 = diag_dominant_bcsr(50, 8, seed=8)
    A8 = bm.Matrix.from_bcsr(rp8, c8, v8, 8)
    with pytest.raises(bm.BmfpError) as e:
        bm.Solver(A8, "fp64", launch_mode="persistent")
    assert e.value.status == bm.ERROR_NOT_SUPPORTED


def test_grid_barrier_wait_runs_out_and_reports(lib, cuda):
    """The persistent kernel's bounded barrier wait, run out on purpose: a
    grid barrier waiting for one CTA more than the grid holds gives up after
    its limit, records the fault the solver's host loop turns into
    BMFP_ERROR_TIMEOUT, and the context stays usable (a persistent solve
    right after it succeeds)."""
    import ctypes
    fault, elapsed = ctypes.c_int(0), ctypes.c_double(0.0)
    st = lib.bmfp_selftest_barrier_timeout(0.05, ctypes.byref(fault), ctypes.byref(elapsed), None)
    assert st == bm.SUCCESS, lib.bmfp_last_error()
    assert fault.value == 1
    assert 0.05 <= elapsed.value < 2.0
    assert lib.bmfp_selftest_barrier_timeout(2.0, None, None, None) == bm.ERROR_INVALID_VALUE
    rp, c, v, b = bm.gen_q4_elasticity(60, 15)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    x, info = bm.Solver(A, "fp64", launch_mode="persistent").solve_host(b)
    assert info["status"] == bm.SUCCESS


def test_auto_launch_mode_takes_the_persistent_kernel_from_a_million_rows(lib, cuda):
    """A 1 000 000-row system under the auto launch mode runs the persistent
    kernel (its bits equal the explicit persistent launch's and, on the same
    grid of 3 CTAs per SM, the graph's); a system just below runs graphs
    (its bits equal the graph launch's at the default grid)."""
    rp, c, v, b = bm.gen_q4_elasticity(1000, 500)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    out = {}
    for mode in ("auto", "persistent", "graph"):
        s = bm.Solver(A, "fp64", launch_mode=mode, ctas_per_sm=3, max_iters=200)
        out[mode] = s.solve_host(b)
        s.close()
    assert out["auto"][1]["iterations"] == 200
    assert _same_bits(out["auto"][0], out["persistent"][0]) and _same_bits(out["auto"][0], out["graph"][0])
    A.close()
    rp, c, v, b = bm.gen_q4_elasticity(999, 500)  # 999 000 rows
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    xa, _ = bm.Solver(A, "fp64", max_iters=100).solve_host(b)
    xg, _ = bm.Solver(A, "fp64", launch_mode="graph", max_iters=100).solve_host(b)
    xp, _ = bm.Solver(A, "fp64", launch_mode="persistent", max_iters=100).solve_host(b)
    assert _same_bits(xa, xg)
    assert not _same_bits(xa, xp)  # the persistent kernel's 3 CTAs per SM sum in another order
    A.close()


def test_concurrent_persistent_solves_on_separate_streams(lib, cuda):
    """Three persistent solves of a 1 000 000-row system launched at once from
    three host threads on three streams: cooperative launches that cannot be
    resident together run one after another (no barrier gives up), and each
    result has the bits of the same solve run alone."""
    import threading
    import torch
    rp, c, v, b = bm.gen_q4_elasticity(1000, 500)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    d_b = dev(b)
    solo = torch.empty_like(d_b)
    bm.Solver(A, "fp64", launch_mode="persistent", max_iters=160).solve(d_b, solo)
    torch.cuda.synchronize()
    out = {}

    def worker(k):
        st = torch.cuda.Stream()
        x = torch.empty_like(d_b)
        s = bm.Solver(A, "fp64", launch_mode="persistent", max_iters=160, stream=st.cuda_stream)
        out[k] = (s.solve(d_b, x, stream=st.cuda_stream), x)
        st.synchronize()

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert len(out) == 3
    for info, x in out.values():
        assert info["status"] == bm.ERROR_NOT_CONVERGED and info["iterations"] == 160, info  # the cap
        assert torch.equal(x.view(torch.int64), solo.view(torch.int64))
    A.close()
