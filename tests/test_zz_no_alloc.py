"""The allocation-free BiCGStab entry point against the allocating solver.

bmfp_bicgstab_solve_noalloc serves callers that cannot call cudaMalloc (a
memory pool or budget that forbids new allocations, real-time loops, plug-ins
whose host owns every allocation): it keeps its Krylov vectors in a fixed
device array inside the library. These tests call it through the C ABI twice
in a row — the second call must not be disturbed by what the first left in
the shared array — and compare each solution with bmfp_solver_solve (stopping
on the same recursive-residual rule) within the solver tests' tolerance, for
FP64 and FP32 values, BCSR (bs 2 and 3) and CSR (bs = 0) input, a values
pointer that is not 16-byte aligned, and a system of exactly the 131 072-row
limit. The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm

pytestmark = pytest.mark.gpu

TOL = 1e-10
MAX_ROWS = 131072


def _solve_noalloc(lib, dtype, rp_d, c_d, v_ptr, nbr, bs, nnzb, d_b, d_x, precond, tol=TOL):
    import torch
    it = ctypes.c_int(0)
    rel = ctypes.c_double(0.0)
    st = lib.bmfp_bicgstab_solve_noalloc(dtype, nbr, bs, nnzb, rp_d.data_ptr(), c_d.data_ptr(), v_ptr,
                                         d_b.data_ptr(), d_x.data_ptr(), tol, 20000, precond,
                                         ctypes.byref(it), ctypes.byref(rel),
                                         torch.cuda.current_stream().cuda_stream)
    return st, it.value, rel.value


def _diag_dominant(nbr, bs, seed, extra=6):
    """Random BCSR with a dominant diagonal block per block row (vectorised)."""
    rng = np.random.default_rng(seed)
    offs = rng.integers(-12, 13, size=(nbr, extra))
    cand = np.clip(np.arange(nbr)[:, None] + np.concatenate([np.zeros((nbr, 1), int), offs], axis=1), 0, nbr - 1)
    rows = [np.unique(r) for r in cand]
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    c = np.concatenate(rows).astype(np.int32)
    v = rng.uniform(-1, 1, (c.size, bs, bs))
    diag = np.repeat(np.arange(nbr), np.diff(rp)) == c
    v[diag] += np.eye(bs) * (extra + 1) * bs * 1.5
    return rp, c, v.reshape(-1)


def _check_pair(lib, A, rp, c, v, nbr, bs, nnzb, rhs_list, precision, dtype, precond=bm.PRECOND_NONE,
                tol=TOL, value_offset=0, same_path=True):
    """Two no-alloc calls in a row, each against bmfp_solver_solve."""
    import torch
    tdt = torch.float64 if dtype == bm.R64F else torch.float32
    solver = bm.Solver(A, precision, tol=tol, max_iters=20000, check_true_residual=False,
                       preconditioner=precond)
    rp_d, c_d = torch.from_numpy(rp).cuda(), torch.from_numpy(c).cuda()
    v_t = torch.from_numpy(np.asarray(v)).to(tdt)
    v_d = torch.zeros(v_t.numel() + value_offset, dtype=tdt, device="cuda")
    v_d[value_offset:] = v_t.cuda()
    v_ptr = v_d.data_ptr() + value_offset * v_d.element_size()
    for b in rhs_list:
        d_b = torch.from_numpy(np.asarray(b)).to(tdt).cuda()
        x_ref = torch.empty_like(d_b)
        info = solver.solve(d_b, x_ref)
        assert info["status"] == bm.SUCCESS, info
        x_na = torch.full_like(d_b, float("nan"))
        st, iters, rel = _solve_noalloc(lib, dtype, rp_d, c_d, v_ptr, nbr, bs, nnzb, d_b, x_na, precond, tol)
        assert st == bm.SUCCESS, lib.bmfp_last_error()
        assert rel < tol
        xa, xr = x_na.double().cpu().numpy(), x_ref.double().cpu().numpy()
        assert np.isfinite(xa).all()
        if same_path:
            # the same phase kernels on the same grid: the same iterations
            assert iters == info["iterations"]
            assert np.linalg.norm(xa - xr) <= tol * np.linalg.norm(xr)
        else:
            # another row routine (scalar loads): another summation order,
            # both within the solve's accuracy on a well-conditioned matrix
            assert abs(iters - info["iterations"]) <= 0.25 * info["iterations"] + 3
            assert np.linalg.norm(xa - xr) <= 1e-8 * np.linalg.norm(xr)
    solver.close()


@pytest.mark.parametrize("precond", [bm.PRECOND_NONE, bm.PRECOND_JACOBI])
def test_noalloc_matches_allocating_solver_on_two_calls(lib, cuda, precond):
    nx, ny = 40, 10
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    rhs2 = np.random.default_rng(11).uniform(-1, 1, rhs.size)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    _check_pair(lib, A, rp, c, v, nx * ny, 2, c.size, (rhs, rhs2), "fp64", bm.R64F, precond)
    A.close()


def test_noalloc_fp32(lib, cuda):
    rp, c, v = _diag_dominant(3000, 2, seed=1)
    rng = np.random.default_rng(2)
    rhs = [rng.uniform(-1, 1, 6000).astype(np.float32) for _ in range(2)]
    v32 = v.astype(np.float32)
    A = bm.Matrix.from_bcsr(rp, c, v32, 2)
    _check_pair(lib, A, rp, c, v32, 3000, 2, c.size, rhs, "fp32", bm.R32F, tol=1e-5)
    A.close()


def test_noalloc_csr_input(lib, cuda):
    """bs = 0: CSR arrays with n_block_rows = rows and nnzb = entries."""
    rp, c, v, rhs = bm.gen_q4_elasticity(30, 8)
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    n = len(crp) - 1
    A = bm.Matrix.from_csr(crp, cc, cv, n)
    rhs2 = np.random.default_rng(3).uniform(-1, 1, n)
    for pre in (bm.PRECOND_NONE, bm.PRECOND_JACOBI):
        _check_pair(lib, A, crp, cc, cv, n, 0, cc.size, (rhs, rhs2), "fp64", bm.R64F, pre)
    A.close()


def test_noalloc_block_size_3(lib, cuda):
    rp, c, v = _diag_dominant(700, 3, seed=4)
    rng = np.random.default_rng(5)
    A = bm.Matrix.from_bcsr(rp, c, v, 3)
    _check_pair(lib, A, rp, c, v, 700, 3, c.size, [rng.uniform(-1, 1, 2100) for _ in range(2)], "fp64", bm.R64F)
    A.close()


def test_noalloc_unaligned_values_take_the_scalar_routine(lib, cuda):
    """A values pointer one element past a 16-byte boundary: the vectorised
    bs-2 routine needs aligned values, so the entry point runs the scalar one."""
    rp, c, v = _diag_dominant(2500, 2, seed=6)
    rng = np.random.default_rng(7)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    _check_pair(lib, A, rp, c, v, 2500, 2, c.size, [rng.uniform(-1, 1, 5000) for _ in range(2)], "fp64",
                bm.R64F, value_offset=1, same_path=False)
    A.close()


def test_noalloc_at_exactly_its_row_limit(lib, cuda):
    nbr = MAX_ROWS // 2
    rp, c, v = _diag_dominant(nbr, 2, seed=8)
    rng = np.random.default_rng(9)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    _check_pair(lib, A, rp, c, v, nbr, 2, c.size, [rng.uniform(-1, 1, MAX_ROWS) for _ in range(2)], "fp64",
                bm.R64F)
    A.close()


def test_noalloc_rejects_systems_over_its_limit(lib, cuda):
    import torch
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    idx = torch.zeros(4, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for nbr, bs in ((70000, 2), (MAX_ROWS + 1, 1), (MAX_ROWS + 1, 0)):
        st = lib.bmfp_bicgstab_solve_noalloc(bm.R64F, nbr, bs, 1, idx.data_ptr(), idx.data_ptr(),
                                             dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), TOL, 10, 0,
                                             None, None, stream)
        assert st == bm.ERROR_NOT_SUPPORTED
        assert b"131072" in lib.bmfp_last_error()
    # more stored values than 32-bit offsets reach (nnzb * bs^2 > 2^31 - 1)
    st = lib.bmfp_bicgstab_solve_noalloc(bm.R64F, 1000, 32, 2200000, idx.data_ptr(), idx.data_ptr(),
                                         dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), TOL, 10, 0,
                                         None, None, stream)
    assert st == bm.ERROR_NOT_SUPPORTED
