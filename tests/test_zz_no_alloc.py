"""The allocation-free BiCGStab entry point against the allocating solver.

bmfp_bicgstab_solve_noalloc serves callers that cannot call cudaMalloc (a
memory pool or budget that forbids new allocations, real-time loops, plug-ins
whose host owns every allocation): it keeps its Krylov vectors in a fixed
device array inside the library. This test calls it through the C ABI twice in
a row — the second call must not be disturbed by what the first left in the
shared array — and compares each solution with bmfp_solver_solve (stopping on
the same recursive-residual rule) within the solver tests' tolerance. The
file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _solve_noalloc(lib, rp_d, c_d, v_d, nbr, bs, nnzb, d_b, d_x, precond):
    import torch
    it = ctypes.c_int(0)
    rel = ctypes.c_double(0.0)
    st = lib.bmfp_bicgstab_solve_noalloc(bm.R64F, nbr, bs, nnzb, rp_d.data_ptr(), c_d.data_ptr(), v_d.data_ptr(),
                                         d_b.data_ptr(), d_x.data_ptr(), TOL, 20000, precond,
                                         ctypes.byref(it), ctypes.byref(rel),
                                         torch.cuda.current_stream().cuda_stream)
    return st, it.value, rel.value


@pytest.mark.parametrize("precond", [bm.PRECOND_NONE, bm.PRECOND_JACOBI])
def test_noalloc_matches_allocating_solver_on_two_calls(lib, cuda, precond):
    import torch
    nx, ny = 40, 10
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    rhs2 = np.random.default_rng(11).uniform(-1, 1, rhs.size)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    solver = bm.Solver(A, "fp64", tol=TOL, max_iters=20000, check_true_residual=False,
                       preconditioner=precond)
    rp_d, c_d, v_d = (torch.from_numpy(a).cuda() for a in (rp, c, v))
    for b in (rhs, rhs2):
        d_b = torch.from_numpy(b).cuda()
        x_ref = torch.empty_like(d_b)
        info = solver.solve(d_b, x_ref)
        assert info["status"] == bm.SUCCESS, info
        x_na = torch.full_like(d_b, float("nan"))
        st, iters, rel = _solve_noalloc(lib, rp_d, c_d, v_d, nx * ny, 2, c.size, d_b, x_na, precond)
        assert st == bm.SUCCESS, lib.bmfp_last_error()
        assert rel < TOL and iters == info["iterations"]
        xa, xr = x_na.cpu().numpy(), x_ref.cpu().numpy()
        assert np.isfinite(xa).all()
        assert np.linalg.norm(xa - xr) <= TOL * np.linalg.norm(xr)
    solver.close()
    A.close()


def test_noalloc_rejects_systems_over_its_limit(lib, cuda):
    import torch
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    idx = torch.zeros(4, dtype=torch.int32, device="cuda")
    st = lib.bmfp_bicgstab_solve_noalloc(bm.R64F, 70000, 2, 1, idx.data_ptr(), idx.data_ptr(), dummy.data_ptr(),
                                         dummy.data_ptr(), dummy.data_ptr(), TOL, 10, 0, None, None,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == bm.ERROR_NOT_SUPPORTED
    assert b"131072" in lib.bmfp_last_error()
