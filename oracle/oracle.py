"""CPU oracle for the block-sparse hot path — TEST INFRASTRUCTURE ONLY.

numpy front end over ``liborc.so`` (the C restatement in ``oracle.c``) plus
independent numpy restatements of the workload generators that have no
reference counterpart (the seeded band generator and the Q4 plane-stress
assembler). Only the test suite, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product never does.

Reference anchors (paths inside gevtushenko/block_matrix_format_performance):
  csr_spmv            main.cpp:36-45
  bcsr_to_csr         common/matrix_converters.h:88-117
  transpose_blocks    common/matrix_converters.h:32-49
  gen_n_diag_bcsr     common/matrix_converters.h:157-196
  compare_results     common/measurement_class.h:58-87
  bicgstab            gpu/bicgstab.cu:387-526 (last iterate returned)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build():
    """Compile liborc.so with the committed Makefile (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for t, p in (("f64", _f64p), ("f32", _f32p)):
            getattr(L, f"orc_csr_spmv_{t}").argtypes = [ctypes.c_int, _i32p, _i32p, p, p, p]
            getattr(L, f"orc_csr_spmv_mt_{t}").argtypes = [ctypes.c_int, _i32p, _i32p, p, p, p, ctypes.c_int]
            getattr(L, f"orc_bcsr_spmv_{t}").argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, p, p, p]
            getattr(L, f"orc_bcsr_to_csr_{t}").argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, p, _i32p, _i32p, p]
            getattr(L, f"orc_csr_to_bcsr_fill_{t}").argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, p, _i32p, _i32p, p]
            getattr(L, f"orc_csr_to_bcsr_fill_{t}").restype = ctypes.c_int
            getattr(L, f"orc_transpose_blocks_{t}").argtypes = [ctypes.c_int, ctypes.c_int, _i32p, p, p]
            getattr(L, f"orc_gen_n_diag_bcsr_{t}").argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, p]
            getattr(L, f"orc_compare_results_{t}").argtypes = [ctypes.c_uint, p, p, ctypes.POINTER(ctypes.c_int)]
            getattr(L, f"orc_compare_results_{t}").restype = ctypes.c_double
        L.orc_csr_to_bcsr_count.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p]
        L.orc_csr_to_bcsr_count.restype = ctypes.c_int64
        L.orc_bicgstab_f64.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_double)]
        L.orc_bicgstab_f64.restype = ctypes.c_int
        L.orc_bicgstab_mt_f64.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double)]
        L.orc_bicgstab_mt_f64.restype = ctypes.c_int
        L.orc_block_jacobi_f64.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f64p, _f64p]
        L.orc_bicgstab_bj_f64.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                          ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_double)]
        L.orc_bicgstab_bj_f64.restype = ctypes.c_int
        L.orc_band_blocks.argtypes = [ctypes.c_int] * 4
        L.orc_band_blocks.restype = ctypes.c_int
        L.orc_gen_band.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                   ctypes.c_int, ctypes.c_int, np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS"),
                                   _i32p, ctypes.c_void_p, ctypes.c_int]
        L.orc_gen_uniform_vector.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                             ctypes.c_void_p]
        _LIB = L
    return _LIB


def _tag(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float64:
        return "f64"
    if dtype == np.float32:
        return "f32"
    raise TypeError(dtype)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ------------------------------------------------------------------- SpMV ---

def csr_spmv(row_ptr, cols, vals, x, threads=1, out=None):
    """y = A x over CSR in the reference loop order (main.cpp:36-45); `out`
    (n elements of the value type) receives y when given."""
    vals = np.ascontiguousarray(vals)
    t = _tag(vals.dtype)
    row_ptr = _c(row_ptr, np.int32)
    n = row_ptr.size - 1
    y = np.zeros(n, dtype=vals.dtype) if out is None else out
    assert y.dtype == vals.dtype and y.size == n and y.flags.c_contiguous
    x = _c(x, vals.dtype)
    if threads > 1:
        getattr(lib(), f"orc_csr_spmv_mt_{t}")(n, row_ptr, _c(cols, np.int32), vals, x, y, threads)
    else:
        getattr(lib(), f"orc_csr_spmv_{t}")(n, row_ptr, _c(cols, np.int32), vals, x, y)
    return y


def bcsr_spmv(row_ptr, cols, vals, bs, x):
    """y = A x over row-major BCSR; bit-identical to csr_spmv(bcsr_to_csr(...))."""
    vals = np.ascontiguousarray(vals)
    t = _tag(vals.dtype)
    row_ptr = _c(row_ptr, np.int32)
    nbr = row_ptr.size - 1
    y = np.zeros(nbr * bs, dtype=vals.dtype)
    getattr(lib(), f"orc_bcsr_spmv_{t}")(nbr, bs, row_ptr, _c(cols, np.int32), vals.reshape(-1),
                                         _c(x, vals.dtype), y)
    return y


def abs_row_sums(row_ptr, cols, vals, x):
    """sum_j |a_ij x_j| per row, in float64 — the scale of the per-entry bound."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    a = np.abs(np.asarray(vals, dtype=np.float64)) * np.abs(np.asarray(x, dtype=np.float64)[np.asarray(cols)])
    cs = np.concatenate([[0.0], np.cumsum(a)])
    return cs[row_ptr[1:]] - cs[row_ptr[:-1]]


# ------------------------------------------------------------ conversions ---

def bcsr_to_csr(row_ptr, cols, vals, bs):
    """common/matrix_converters.h:88-117."""
    vals = np.ascontiguousarray(vals).reshape(-1)
    t = _tag(vals.dtype)
    row_ptr = _c(row_ptr, np.int32)
    nbr = row_ptr.size - 1
    nnz = int(row_ptr[-1]) * bs * bs
    o_rp = np.zeros(nbr * bs + 1, np.int32)
    o_c = np.zeros(nnz, np.int32)
    o_v = np.zeros(nnz, vals.dtype)
    getattr(lib(), f"orc_bcsr_to_csr_{t}")(nbr, bs, row_ptr, _c(cols, np.int32), vals, o_rp, o_c, o_v)
    return o_rp, o_c, o_v


def csr_to_bcsr(row_ptr, cols, vals, n_cols, bs):
    """Inverse of bcsr_to_csr: explicit zeros fill each touched block."""
    vals = np.ascontiguousarray(vals)
    t = _tag(vals.dtype)
    row_ptr = _c(row_ptr, np.int32)
    cols = _c(cols, np.int32)
    n_rows = row_ptr.size - 1
    if n_rows % bs:
        raise ValueError("rows not a multiple of bs")
    brp = np.zeros(n_rows // bs + 1, np.int32)
    nnzb = lib().orc_csr_to_bcsr_count(n_rows, n_cols, bs, row_ptr, cols, brp)
    if nnzb < 0:
        raise ValueError("invalid CSR for this block size")
    bc = np.zeros(nnzb, np.int32)
    bv = np.zeros(nnzb * bs * bs, vals.dtype)
    rc = getattr(lib(), f"orc_csr_to_bcsr_fill_{t}")(n_rows, bs, row_ptr, cols, vals, brp, bc, bv)
    if rc != 0:
        raise ValueError("conversion failed")
    return brp, bc, bv


def transpose_blocks(row_ptr, vals, bs):
    """common/matrix_converters.h:32-49."""
    vals = np.ascontiguousarray(vals).reshape(-1)
    t = _tag(vals.dtype)
    row_ptr = _c(row_ptr, np.int32)
    out = np.empty_like(vals)
    getattr(lib(), f"orc_transpose_blocks_{t}")(row_ptr.size - 1, bs, row_ptr, vals, out)
    return out


def gen_n_diag_bcsr(n_rows, blocks_per_row, bs, dtype=np.float64):
    """common/matrix_converters.h:157-196."""
    t = _tag(dtype)
    rp = np.zeros(n_rows + 1, np.int32)
    c = np.zeros(n_rows * blocks_per_row, np.int32)
    v = np.zeros(n_rows * blocks_per_row * bs * bs, dtype)
    getattr(lib(), f"orc_gen_n_diag_bcsr_{t}")(n_rows, blocks_per_row, bs, rp, c, v)
    return rp, c, v


def compare_results(a, b):
    """common/measurement_class.h:58-87 -> (error, flagged)."""
    a = np.ascontiguousarray(a)
    t = _tag(a.dtype)
    flag = ctypes.c_int(0)
    err = getattr(lib(), f"orc_compare_results_{t}")(a.size, a, _c(b, a.dtype), ctypes.byref(flag))
    return err, bool(flag.value)


def bicgstab(row_ptr, cols, vals, b, eps, max_iterations, use_precond=False):
    """gpu/bicgstab.cu:387-526 recurrences on the CPU -> (x, status, iters, rel_res)."""
    row_ptr = _c(row_ptr, np.int32)
    n = row_ptr.size - 1
    x = np.zeros(n, np.float64)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0)
    st = lib().orc_bicgstab_f64(n, row_ptr, _c(cols, np.int32), _c(vals, np.float64), _c(b, np.float64), x,
                                float(eps), int(max_iterations), int(bool(use_precond)),
                                ctypes.byref(it), ctypes.byref(rr))
    return x, st, it.value, rr.value


# -------------------------------------------- generators (restated specs) ---

_M64 = (1 << 64) - 1


def block_jacobi(row_ptr, cols, vals, bs):
    """Inverses of the bs x bs diagonal blocks of a CSR matrix (identity where
    singular), shape (n/bs, bs, bs)."""
    row_ptr = _c(row_ptr, np.int32)
    n = row_ptr.size - 1
    out = np.zeros(n * bs, np.float64)
    lib().orc_block_jacobi_f64(n, bs, row_ptr, _c(cols, np.int32), _c(vals, np.float64), out)
    return out.reshape(-1, bs, bs)


def bicgstab_block_jacobi(row_ptr, cols, vals, bs, b, eps, max_iterations):
    """bicgstab with block-Jacobi right preconditioning -> (x, status, iters, rel_res)."""
    row_ptr = _c(row_ptr, np.int32)
    n = row_ptr.size - 1
    x = np.zeros(n, np.float64)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0)
    st = lib().orc_bicgstab_bj_f64(n, bs, row_ptr, _c(cols, np.int32), _c(vals, np.float64), _c(b, np.float64), x,
                                   float(eps), int(max_iterations), ctypes.byref(it), ctypes.byref(rr))
    return x, st, it.value, rr.value


def bicgstab_mt(row_ptr, cols, vals, b, eps, max_iterations, threads, use_precond=False):
    """bicgstab's recurrences on `threads` host threads (the CPU solve
    baseline on all cores). Returns (x, status, iterations, rel residual)."""
    b = _c(b, np.float64)
    x = np.zeros_like(b)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0.0)
    st = lib().orc_bicgstab_mt_f64(b.size, _c(row_ptr, np.int32), _c(cols, np.int32), _c(vals, np.float64), b, x,
                                   eps, max_iterations, int(use_precond), threads, ctypes.byref(it),
                                   ctypes.byref(rr))
    return x, st, it.value, rr.value


def _splitmix64(state):
    """SplitMix64 (Steele, Lea, Flood 2014) over uint64 numpy arrays."""
    with np.errstate(over="ignore"):
        state = (state + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(_M64)
        z = state
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return state, z


def _row_states(seed, stream, rows):
    """Per-row generator state: splitmix64 of (seed, stream, row) mixed."""
    with np.errstate(over="ignore"):
        base = np.uint64(seed & _M64) * np.uint64(0xD1B54A32D192ED03) + np.uint64(stream) * np.uint64(0x8CB92BA72F3D8DD7)
        s = np.asarray(rows, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + base
    _, z = _splitmix64(s)
    return z


def _uniform_pm1(z):
    """Top 53 bits of z -> double in [-1, 1)."""
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def gen_band_bcsr(n_block_rows, blocks_per_row, half_band, bs, seed, dtype=np.float64):
    """Seeded random-band BCSR: for block row i, min(k, W) distinct block
    columns from [max(0,i-h), min(nbr-1,i+h)] (W wide) by a partial
    Fisher-Yates shuffle driven by per-row SplitMix64 streams, sorted; values
    U[-1,1) drawn per block row in storage order (stream 1), rounded to dtype.
    Independent restatement of the product generator's specification."""
    nbr = n_block_rows
    rows = np.arange(nbr, dtype=np.int64)
    lo = np.maximum(0, rows - half_band)
    hi = np.minimum(nbr - 1, rows + half_band)
    W = hi - lo + 1
    k = np.minimum(blocks_per_row, W)
    kmax = int(k.max()) if nbr else 0
    wmax = int(W.max()) if nbr else 0
    perm = np.tile(np.arange(wmax, dtype=np.int64), (nbr, 1))
    st = _row_states(seed, 0, rows)
    for j in range(kmax):
        st, z = _splitmix64(st)
        active = j < k
        span = np.maximum(W - j, 1).astype(np.uint64)
        pick = j + (z % span).astype(np.int64)
        a = perm[rows, j].copy()
        bpk = perm[rows, np.where(active, pick, j)]
        perm[rows, j] = np.where(active, bpk, a)
        perm[rows, np.where(active, pick, j)] = np.where(active, a, bpk)
    row_ptr = np.zeros(nbr + 1, np.int64)
    row_ptr[1:] = np.cumsum(k)
    cols = np.empty(int(row_ptr[-1]), np.int64)
    for j in range(kmax):
        sel = j < k
        cols[row_ptr[:-1][sel] + j] = perm[sel, j] + lo[sel]
    for i in range(nbr):  # per-row sort (small k)
        cols[row_ptr[i]:row_ptr[i + 1]].sort()
    # values: per block row, bs*bs*k draws from stream 1
    nvals_row = k * bs * bs
    vals = np.empty(int(row_ptr[-1]) * bs * bs, np.float64)
    vst = _row_states(seed, 1, rows)
    vmax = int(nvals_row.max()) if nbr else 0
    voff = row_ptr[:-1] * bs * bs
    for j in range(vmax):
        vst, z = _splitmix64(vst)
        sel = j < nvals_row
        vals[voff[sel] + j] = _uniform_pm1(z[sel])
    return row_ptr.astype(np.int32), cols.astype(np.int32), vals.astype(dtype)


def gen_uniform_vector(n, seed, stream, dtype=np.float64):
    """x_i = U[-1,1) from splitmix64 of (seed, stream, i)."""
    z = _row_states(seed, stream, np.arange(n, dtype=np.int64))
    return _uniform_pm1(z).astype(dtype)


def band_block_counts(n_block_rows, blocks_per_row, half_band):
    """Blocks per block row of the seeded band workload: min(k, band width)."""
    rows = np.arange(n_block_rows, dtype=np.int64)
    w = np.minimum(n_block_rows - 1, rows + half_band) - np.maximum(0, rows - half_band) + 1
    return np.minimum(blocks_per_row, w)


def gen_band_c(n_block_rows, blocks_per_row, half_band, bs, seed, dtype=np.float64, csr=False, threads=1):
    """The band generator of oracle.c (the specification of gen_band_bcsr
    above, in C, threaded over block rows): BCSR (row_ptr, cols, vals) or,
    with csr=True, its CSR expansion (the reference CPU loop's input) without
    the BCSR intermediate."""
    k = band_block_counts(n_block_rows, blocks_per_row, half_band)
    if csr:
        rp64 = np.zeros(n_block_rows * bs + 1, np.int64)
        np.cumsum(np.repeat(k * bs, bs), out=rp64[1:])
    else:
        rp64 = np.zeros(n_block_rows + 1, np.int64)
        np.cumsum(k, out=rp64[1:])
    if rp64[-1] > np.iinfo(np.int32).max:
        raise ValueError("offsets exceed 32 bits")
    # CSR: rp64[-1] scalar entries; BCSR: rp64[-1] blocks of bs*bs values
    cols = np.empty(int(rp64[-1]), np.int32)
    vals = np.empty(int(rp64[-1]) * (1 if csr else bs * bs), np.dtype(dtype))
    lib().orc_gen_band(n_block_rows, blocks_per_row, half_band, bs, seed, int(np.dtype(dtype) == np.float64),
                       int(csr), rp64, cols, vals.ctypes.data, threads)
    return rp64.astype(np.int32), cols, vals


def gen_uniform_vector_c(n, seed, stream, dtype=np.float64):
    """gen_uniform_vector in C."""
    out = np.empty(n, np.dtype(dtype))
    lib().orc_gen_uniform_vector(n, seed, stream, int(np.dtype(dtype) == np.float64), out.ctypes.data)
    return out


def q4_element_stiffness(E=1.0, nu=0.3, t=1.0, hx=1.0, hy=1.0):
    """Bilinear quad plane-stress stiffness (8x8, DOFs (ux,uy) per node in
    counter-clockwise order from the lower-left corner) by 2x2 Gauss."""
    D = E / (1.0 - nu * nu) * np.array([[1.0, nu, 0.0], [nu, 1.0, 0.0], [0.0, 0.0, (1.0 - nu) / 2.0]])
    g = 1.0 / np.sqrt(3.0)
    xi_n = np.array([-1.0, 1.0, 1.0, -1.0])
    eta_n = np.array([-1.0, -1.0, 1.0, 1.0])
    K = np.zeros((8, 8))
    for xi in (-g, g):
        for eta in (-g, g):
            dN_dxi = 0.25 * xi_n * (1.0 + eta * eta_n)
            dN_deta = 0.25 * eta_n * (1.0 + xi * xi_n)
            dN_dx = dN_dxi * (2.0 / hx)
            dN_dy = dN_deta * (2.0 / hy)
            B = np.zeros((3, 8))
            B[0, 0::2] = dN_dx
            B[1, 1::2] = dN_dy
            B[2, 0::2] = dN_dy
            B[2, 1::2] = dN_dx
            K += B.T @ D @ B * (hx * hy / 4.0) * t
    return K


def q4_elasticity_dense(nx, ny, E=1.0, nu=0.3):
    """Dense assembled operator and load for small grids (nx*ny nodes): left
    column clamped (identity rows/columns), f_y = -1 on right-edge nodes."""
    n = 2 * nx * ny
    K = np.zeros((n, n))
    ke = q4_element_stiffness(E, nu)
    for j in range(ny - 1):
        for i in range(nx - 1):
            nodes = [j * nx + i, j * nx + i + 1, (j + 1) * nx + i + 1, (j + 1) * nx + i]
            dofs = np.array([[2 * a, 2 * a + 1] for a in nodes]).reshape(-1)
            K[np.ix_(dofs, dofs)] += ke
    clamped = np.zeros(n, bool)
    for j in range(ny):
        clamped[2 * (j * nx)] = clamped[2 * (j * nx) + 1] = True
    K[clamped, :] = 0.0
    K[:, clamped] = 0.0
    K[clamped, clamped] = 1.0
    f = np.zeros(n)
    for j in range(ny):
        f[2 * (j * nx + nx - 1) + 1] = -1.0
    return K, f
