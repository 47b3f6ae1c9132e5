"""GB300-native block-sparse SpMV and BiCGStab — Python front end.

The product is ``libbmfp.so`` (CUDA kernels for sm_103a behind the C ABI in
``include/bmfp.h``) and the C++ headers in ``include/bmfp/`` that rebuild the
reference's host API. This module is a thin ctypes layer used by the tests and
the benchmark: numpy arrays for host data, torch CUDA tensors for device
memory and streams. Every device call goes through the C ABI; there is no
Python or CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._capi import (BmfpError, ServerOptions, ServerStats, SolveInfo, SolverOptions, check, load,  # noqa: F401
                    LIB_PATH)

R32F, R64F = 0, 1

# enum bmfp_spmv_variant (include/bmfp.h)
CSR_SCALAR, CSR_VECTOR, CSR_NATIVE = 0, 1, 2
BCSR_ROW_THREAD, BCSR_ROW_WARP = 3, 4
BCSR_COL_THREAD, BCSR_COL_THREAD_TEMPLATE = 5, 6
BCSR_COL_COAL_X, BCSR_COL_COAL_X_TEMPLATE = 7, 8
BCSR_COL_BY_COL, BCSR_COL_BY_COL_FASTDIV, BCSR_COL_BY_COL_PO2, BCSR_COL_BY_COL_TEMPLATE = 9, 10, 11, 12
BCSR_JIT, CUSPARSE_ROW, CUSPARSE_COL, BCSR_NATIVE = 13, 14, 15, 16
VARIANT_COUNT = 17
LANES_ROW_OWNER, LANES_COL_OWNER = 64, 65

SUCCESS, ERROR_INVALID_VALUE, ERROR_CUDA, ERROR_OUT_OF_MEMORY, ERROR_NOT_SUPPORTED = 0, 1, 2, 3, 4
ERROR_BREAKDOWN, ERROR_NOT_CONVERGED, ERROR_TIMEOUT, ERROR_BUDGET, PENDING = 5, 6, 7, 8, 9


def dtype_enum(dtype) -> int:
    dt = np.dtype(dtype) if not hasattr(dtype, "is_floating_point") else dtype
    name = str(dt).replace("torch.", "")
    if name in ("float64", "double"):
        return R64F
    if name in ("float32", "float"):
        return R32F
    raise TypeError(f"unsupported dtype {dtype}")


def np_dtype(enum: int):
    return np.float64 if enum == R64F else np.float32


def _p(a):
    """Raw pointer of a numpy array, torch tensor or int (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _stream(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except Exception:  # pragma: no cover
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def variant_name(v: int) -> str:
    s = load().bmfp_spmv_variant_name(v)
    return s.decode() if s else None


def variant_layout(v: int) -> int:
    return load().bmfp_spmv_variant_layout(v)


def variant_is_csr(v: int) -> int:
    return load().bmfp_spmv_variant_is_csr(v)


def device_count() -> int:
    return load().bmfp_device_count()


# ----------------------------------------------------------- host utilities

def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def gen_n_diag_bcsr(n_rows, blocks_per_row, bs, dtype=np.float64):
    """The reference's band generator (common/matrix_converters.h:157-196)."""
    L = load()
    rp = np.zeros(n_rows + 1, np.int32)
    c = np.zeros(n_rows * blocks_per_row, np.int32)
    v = np.zeros(n_rows * blocks_per_row * bs * bs, dtype)
    check(L.bmfp_gen_n_diag_bcsr(dtype_enum(dtype), n_rows, blocks_per_row, bs, _p(rp), _p(c), _p(v)))
    return rp, c, v


def gen_band_bcsr(n_block_rows, blocks_per_row, half_band, bs, seed, dtype=np.float64):
    """Seeded random-band BCSR (the block-size sweep workload)."""
    L = load()
    e = dtype_enum(dtype)
    rp = np.zeros(n_block_rows + 1, np.int32)
    nnzb = ctypes.c_int64(0)
    check(L.bmfp_gen_band_bcsr(e, n_block_rows, blocks_per_row, half_band, bs, seed, _p(rp),
                               ctypes.byref(nnzb), None, None))
    c = np.zeros(nnzb.value, np.int32)
    v = np.zeros(nnzb.value * bs * bs, dtype)
    check(L.bmfp_gen_band_bcsr(e, n_block_rows, blocks_per_row, half_band, bs, seed, _p(rp),
                               ctypes.byref(nnzb), _p(c), _p(v)))
    return rp, c, v


def gen_uniform_vector(n, seed, stream, dtype=np.float64):
    out = np.zeros(n, dtype)
    check(load().bmfp_gen_uniform_vector(dtype_enum(dtype), n, seed, stream, _p(out)))
    return out


def gen_q4_elasticity(nx, ny, dtype=np.float64, young=1.0, poisson=0.3):
    """Q4 plane-stress stiffness (BCSR bs=2) and load for an nx*ny node grid."""
    L = load()
    e = dtype_enum(dtype)
    rp = np.zeros(nx * ny + 1, np.int32)
    nnzb = ctypes.c_int64(0)
    check(L.bmfp_gen_q4_elasticity(e, nx, ny, young, poisson, _p(rp), ctypes.byref(nnzb), None, None, None))
    c = np.zeros(nnzb.value, np.int32)
    v = np.zeros(nnzb.value * 4, dtype)
    rhs = np.zeros(2 * nx * ny, dtype)
    check(L.bmfp_gen_q4_elasticity(e, nx, ny, young, poisson, _p(rp), ctypes.byref(nnzb), _p(c), _p(v),
                                   _p(rhs)))
    return rp, c, v, rhs


def gen_golden_gate_bridge(main_span=1280.0, side_span=345.0, tower_height=230.0, segment_length=7.62,
                           load_window=450.0, load_fy=-2e6, dtype=np.float64):
    """Truss model of the Golden Gate bridge (bmfp_gen_golden_gate_bridge): BCSR
    bs=2 stiffness (row_ptr, cols, values) and load vector. main.cpp's bridge
    is main_span=128000, tower_height=260."""
    L = load()
    e = dtype_enum(dtype)
    args = (float(main_span), float(side_span), float(tower_height), float(segment_length), float(load_window),
            float(load_fy))
    nbr, nnzb = ctypes.c_int(0), ctypes.c_int64(0)
    check(L.bmfp_gen_golden_gate_bridge(e, *args, ctypes.byref(nbr), ctypes.byref(nnzb), None, None, None, None))
    rp = np.zeros(nbr.value + 1, np.int32)
    c = np.zeros(nnzb.value, np.int32)
    v = np.zeros(nnzb.value * 4, dtype)
    rhs = np.zeros(2 * nbr.value, dtype)
    check(L.bmfp_gen_golden_gate_bridge(e, *args, ctypes.byref(nbr), ctypes.byref(nnzb), _p(rp), _p(c), _p(v),
                                        _p(rhs)))
    return rp, c, v, rhs


def bcsr_to_csr(row_ptr, cols, vals, bs):
    vals = np.ascontiguousarray(vals).reshape(-1)
    row_ptr = _i32(row_ptr)
    nbr = row_ptr.size - 1
    nnz = int(row_ptr[-1]) * bs * bs
    rp = np.zeros(nbr * bs + 1, np.int32)
    c = np.zeros(nnz, np.int32)
    v = np.zeros(nnz, vals.dtype)
    check(load().bmfp_bcsr_to_csr(dtype_enum(vals.dtype), nbr, bs, _p(row_ptr), _p(_i32(cols)), _p(vals),
                                  _p(rp), _p(c), _p(v)))
    return rp, c, v


def csr_to_bcsr(row_ptr, cols, vals, n_cols, bs):
    L = load()
    vals = np.ascontiguousarray(vals)
    row_ptr, cols = _i32(row_ptr), _i32(cols)
    n_rows = row_ptr.size - 1
    e = dtype_enum(vals.dtype)
    brp = np.zeros(n_rows // bs + 1, np.int32)
    nnzb = ctypes.c_int64(0)
    check(L.bmfp_csr_to_bcsr(e, n_rows, n_cols, bs, _p(row_ptr), _p(cols), _p(vals), _p(brp),
                             ctypes.byref(nnzb), None, None))
    bc = np.zeros(nnzb.value, np.int32)
    bv = np.zeros(nnzb.value * bs * bs, vals.dtype)
    check(L.bmfp_csr_to_bcsr(e, n_rows, n_cols, bs, _p(row_ptr), _p(cols), _p(vals), _p(brp),
                             ctypes.byref(nnzb), _p(bc), _p(bv)))
    return brp, bc, bv


def mm_read_csr(path, dtype=np.float64):
    """MatrixMarket coordinate file -> (row_ptr, cols, vals, n_cols) through
    bmfp_mm_read_csr; bs-blocked with csr_to_bcsr(row_ptr, cols, vals, n_cols, bs)."""
    m, n, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
    e = dtype_enum(dtype)
    p = os.fsencode(path)
    check(load().bmfp_mm_read_csr(p, e, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), None, None, None))
    rp = np.empty(m.value + 1, np.int32)
    cols = np.empty(nnz.value, np.int32)
    vals = np.empty(nnz.value, np_dtype(e))
    check(load().bmfp_mm_read_csr(p, e, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), _p(rp), _p(cols),
                                  _p(vals)))
    return rp, cols, vals, n.value


def transpose_blocks(row_ptr, vals, bs):
    vals = np.ascontiguousarray(vals).reshape(-1)
    row_ptr = _i32(row_ptr)
    out = np.empty_like(vals)
    check(load().bmfp_transpose_blocks(dtype_enum(vals.dtype), row_ptr.size - 1, bs, _p(row_ptr), _p(vals),
                                       _p(out)))
    return out


def bcsr_spmv_bytes(dtype, n_block_rows, n_block_cols, bs, nnzb) -> int:
    return load().bmfp_bcsr_spmv_bytes(dtype_enum(dtype), n_block_rows, n_block_cols, bs, nnzb)


def csr_spmv_bytes(dtype, n_rows, n_cols, nnz) -> int:
    return load().bmfp_csr_spmv_bytes(dtype_enum(dtype), n_rows, n_cols, nnz)


# ------------------------------------------------------------ device calls

def bcsr_spmv(variant, row_ptr, cols, vals, x, y, bs, n_block_cols=None, stream=None):
    """y = A x through bmfp_bcsr_spmv; arrays are torch CUDA tensors."""
    nbr = row_ptr.numel() - 1
    nbc = n_block_cols if n_block_cols is not None else x.numel() // bs
    check(load().bmfp_bcsr_spmv(dtype_enum(vals.dtype), variant, nbr, nbc, bs, cols.numel(), _p(row_ptr),
                                _p(cols), _p(vals), _p(x), _p(y), _stream(stream)))
    return y


def bcsr_spmv_native(row_ptr, cols, vals, x, y, bs, lanes=0, stream=None):
    check(load().bmfp_bcsr_spmv_native_ex(dtype_enum(vals.dtype), row_ptr.numel() - 1, bs, cols.numel(),
                                          _p(row_ptr), _p(cols), _p(vals), _p(x), _p(y), lanes,
                                          _stream(stream)))
    return y


def bcsr_spmv_colmajor(row_ptr, cols, vals_colmajor, x, y, bs, stream=None):
    """Column-owner product on device arrays with column-major blocks."""
    check(load().bmfp_bcsr_spmv_colmajor(dtype_enum(vals_colmajor.dtype), row_ptr.numel() - 1, bs, cols.numel(),
                                         _p(row_ptr), _p(cols), _p(vals_colmajor), _p(x), _p(y), _stream(stream)))
    return y


def csr_spmv(variant, row_ptr, cols, vals, x, y, n_cols=None, stream=None):
    n = row_ptr.numel() - 1
    check(load().bmfp_csr_spmv(dtype_enum(vals.dtype), variant, n, n_cols if n_cols is not None else x.numel(),
                               cols.numel(), _p(row_ptr), _p(cols), _p(vals), _p(x), _p(y), _stream(stream)))
    return y


def bcsr_spmv_host(row_ptr, cols, vals, x, bs, y=None, n_block_cols=None, lanes=0, stream=None):
    """y = A x with every array in host memory (numpy, ideally views of pinned
    buffers) through bmfp_bcsr_spmv_host: chunked upload overlapped with the
    product, result in y on return. bs = 1 multiplies CSR."""
    vals = np.ascontiguousarray(vals).reshape(-1)
    row_ptr, cols = _i32(row_ptr), _i32(cols)
    x = np.ascontiguousarray(x, dtype=vals.dtype)
    nbr = row_ptr.size - 1
    if y is None:
        y = np.empty(nbr * bs, dtype=vals.dtype)
    assert y.dtype == vals.dtype and y.flags.c_contiguous and y.size == nbr * bs
    nbc = n_block_cols if n_block_cols is not None else x.size // bs
    check(load().bmfp_bcsr_spmv_host(dtype_enum(vals.dtype), nbr, nbc, bs, cols.size, _p(row_ptr), _p(cols),
                                     _p(vals), _p(x), _p(y), lanes, _stream(stream)))
    return y


def measure_fma_peak(dtype=np.float64, stream=None) -> float:
    """FMA throughput of the current GPU in GFLOP/s (bmfp_measure_fma_peak)."""
    g = ctypes.c_double()
    check(load().bmfp_measure_fma_peak(dtype_enum(dtype), ctypes.byref(g), _stream(stream)))
    return g.value


def stream_read(buf, nbytes=None, stream=None) -> None:
    """Launch one plain streaming read of a device tensor (bmfp_stream_read):
    time it like a product to get the size-matched read floor."""
    n = buf.numel() * buf.element_size() if nbytes is None else int(nbytes)
    check(load().bmfp_stream_read(ctypes.c_void_p(buf.data_ptr()), n, _stream(stream)))


def native_default_lanes(dtype, bs, avg_blocks_per_row) -> int:
    return load().bmfp_bcsr_native_default_lanes(dtype_enum(dtype), bs, float(avg_blocks_per_row))


class Matrix:
    """Device-resident matrix handle (bmfp_matrix_t) uploaded from host arrays."""

    def __init__(self, handle, dtype, n_rows, n_cols, bs, nnz):
        self.handle = handle
        self.dtype = dtype
        self.n_rows, self.n_cols, self.bs, self.nnz = n_rows, n_cols, bs, nnz

    @classmethod
    def from_bcsr(cls, row_ptr, cols, vals, bs, n_block_cols=None, dtype=None, stream=None):
        vals = np.ascontiguousarray(vals).reshape(-1)
        if dtype is not None:
            vals = vals.astype(dtype)
        row_ptr, cols = _i32(row_ptr), _i32(cols)
        nbr = row_ptr.size - 1
        nbc = n_block_cols if n_block_cols is not None else nbr
        h = ctypes.c_void_p()
        e = dtype_enum(vals.dtype)
        check(load().bmfp_matrix_create_bcsr(ctypes.byref(h), e, nbr, nbc, bs, cols.size, _p(row_ptr),
                                             _p(cols), _p(vals), _stream(stream)))
        return cls(h, e, nbr, nbc, bs, cols.size)

    @classmethod
    def from_csr(cls, row_ptr, cols, vals, n_cols, stream=None):
        vals = np.ascontiguousarray(vals)
        row_ptr, cols = _i32(row_ptr), _i32(cols)
        h = ctypes.c_void_p()
        e = dtype_enum(vals.dtype)
        check(load().bmfp_matrix_create_csr(ctypes.byref(h), e, row_ptr.size - 1, n_cols, cols.size, _p(row_ptr),
                                            _p(cols), _p(vals), _stream(stream)))
        return cls(h, e, row_ptr.size - 1, n_cols, 0, cols.size)

    def convert(self, dtype, stream=None):
        h = ctypes.c_void_p()
        e = dtype_enum(dtype)
        check(load().bmfp_matrix_convert(ctypes.byref(h), self.handle, e, _stream(stream)))
        return Matrix(h, e, self.n_rows, self.n_cols, self.bs, self.nnz)

    @property
    def rows(self):
        return self.n_rows * (self.bs or 1)

    @property
    def cols(self):
        return self.n_cols * (self.bs or 1)

    def bytes_per_spmv(self) -> int:
        b = ctypes.c_int64(0)
        check(load().bmfp_matrix_info(self.handle, None, None, None, None, None, ctypes.byref(b)))
        return b.value

    def spmv(self, x, y, stream=None):
        check(load().bmfp_matrix_spmv(self.handle, _p(x), _p(y), _stream(stream)))
        return y

    def set_lanes(self, lanes, stream=None):
        """Pin the mapping (LANES_COL_OWNER builds the column-major copy)."""
        check(load().bmfp_matrix_set_lanes(self.handle, lanes, _stream(stream)))

    def autotune(self, x, y, stream=None) -> int:
        g = ctypes.c_int(0)
        check(load().bmfp_matrix_autotune(self.handle, _p(x), _p(y), _stream(stream), ctypes.byref(g)))
        return g.value

    def close(self):
        if self.handle:
            load().bmfp_matrix_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SOLVE_FP64, SOLVE_FP32, SOLVE_MIXED = 0, 1, 2
PRECOND_NONE, PRECOND_JACOBI, PRECOND_BLOCK_JACOBI = 0, 1, 2
LAUNCH_AUTO, LAUNCH_GRAPH, LAUNCH_PERSISTENT = 0, 1, 2
_LAUNCH_MODES = {"auto": LAUNCH_AUTO, "graph": LAUNCH_GRAPH, "persistent": LAUNCH_PERSISTENT}
_PRECISIONS = {"fp64": SOLVE_FP64, "fp32": SOLVE_FP32, "mixed": SOLVE_MIXED}


def solver_options(base=None, **kw) -> SolverOptions:
    """bmfp_solver_options: the library defaults (or `base`), then keyword overrides."""
    o = SolverOptions()
    if base is not None:
        ctypes.pointer(o)[0] = base
    else:
        load().bmfp_solver_options_init(ctypes.byref(o))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = _PRECISIONS[v]
        if k == "preconditioner" and isinstance(v, str):
            v = {"none": PRECOND_NONE, "jacobi": PRECOND_JACOBI, "block_jacobi": PRECOND_BLOCK_JACOBI}[v]
        if k == "launch_mode" and isinstance(v, str):
            v = _LAUNCH_MODES[v]
        setattr(o, k, int(v) if isinstance(v, bool) else v)
    return o


class Solver:
    """bmfp_solver_t: BiCGStab bound to a device matrix handle."""

    def __init__(self, matrix: "Matrix", precision="fp64", tol=1e-10, max_iters=100000, stream=None, **kw):
        self.matrix = matrix
        self.options = solver_options(precision=precision, tolerance=tol, max_iterations=max_iters, **kw)
        h = ctypes.c_void_p()
        check(load().bmfp_solver_create(ctypes.byref(h), matrix.handle, ctypes.byref(self.options),
                                        _stream(stream)))
        self.handle = h

    def solve(self, d_b, d_x, stream=None, raise_on_failure=False) -> dict:
        """Solve A x = b for device vectors; returns bmfp_solve_info as a dict."""
        info = SolveInfo()
        st = load().bmfp_solver_solve(self.handle, _p(d_b), _p(d_x), ctypes.byref(info), _stream(stream))
        if st not in (SUCCESS, ERROR_NOT_CONVERGED, ERROR_BREAKDOWN) or (raise_on_failure and st != SUCCESS):
            check(st)
        return info.as_dict()

    def solve_host(self, b, stream=None):
        """Host numpy right-hand side in, host solution and info out."""
        import torch
        tdt = torch.float64 if self.matrix.dtype == R64F else torch.float32
        d_b = torch.from_numpy(np.ascontiguousarray(b, dtype=np_dtype(self.matrix.dtype))).cuda()
        d_x = torch.empty_like(d_b, dtype=tdt)
        info = self.solve(d_b, d_x, stream)
        return d_x.cpu().numpy(), info

    def close(self):
        if getattr(self, "handle", None):
            load().bmfp_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """bmfp_batch_t: many systems in one persistent, graph-captured launch."""

    def __init__(self, matrices, precision="fp64", tol=1e-10, max_iters=100000, stream=None, **kw):
        self.matrices = list(matrices)
        self.options = solver_options(precision=precision, tolerance=tol, max_iterations=max_iters, **kw)
        n = len(self.matrices)
        arr = (ctypes.c_void_p * max(n, 1))(*[m.handle.value if hasattr(m.handle, "value") else m.handle
                                               for m in self.matrices])
        h = ctypes.c_void_p()
        check(load().bmfp_batch_create(ctypes.byref(h), n, arr, ctypes.byref(self.options), _stream(stream)))
        self.handle = h
        self.n = n

    def _ptrs(self, tensors):
        return (ctypes.c_void_p * max(self.n, 1))(*[_p(t) for t in tensors])

    def configure(self, cluster_size, threads_per_cta):
        check(load().bmfp_batch_configure(self.handle, cluster_size, threads_per_cta))

    def autotune(self, d_bs, d_xs, probe_iterations=16, stream=None):
        c, t = ctypes.c_int(0), ctypes.c_int(0)
        check(load().bmfp_batch_autotune(self.handle, self._ptrs(d_bs), self._ptrs(d_xs), probe_iterations,
                                         ctypes.byref(c), ctypes.byref(t), _stream(stream)))
        return c.value, t.value

    def solve(self, d_bs, d_xs, stream=None):
        infos = (SolveInfo * max(self.n, 1))()
        st = load().bmfp_batch_solve(self.handle, self._ptrs(d_bs), self._ptrs(d_xs), infos, _stream(stream))
        if st not in (SUCCESS, ERROR_NOT_CONVERGED, ERROR_BREAKDOWN):
            check(st)
        return [infos[i].as_dict() for i in range(self.n)]

    def close(self):
        if getattr(self, "handle", None):
            load().bmfp_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """bmfp_server_t: continuous batching of solve requests."""

    def __init__(self, precision="fp64", tol=1e-10, max_iters=100000, hbm_budget_bytes=120 << 30, **kw):
        o = ServerOptions()
        load().bmfp_server_options_init(ctypes.byref(o))
        o.hbm_budget_bytes = hbm_budget_bytes
        for k in ("max_in_flight", "max_batch", "streams", "cluster_size", "threads_per_cta", "wide_threshold_rows",
                  "wide_lanes"):
            if k in kw:
                setattr(o, k, kw.pop(k))
        # start from the server's own solver defaults (one CTA per SM for the whole-GPU lanes)
        o.solver = solver_options(o.solver, precision=precision, tolerance=tol, max_iterations=max_iters, **kw)
        self.options = o
        h = ctypes.c_void_p()
        check(load().bmfp_server_create(ctypes.byref(h), ctypes.byref(o)))
        self.handle = h
        self._keep = {}

    def submit(self, matrix, b, x_out):
        """Queue A x = b (host float64 arrays); x_out is filled on completion."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        t = ctypes.c_uint64(0)
        check(load().bmfp_server_submit(self.handle, matrix.handle, _p(b), _p(x_out), ctypes.byref(t)))
        self._keep[t.value] = (b, x_out)
        return t.value

    def poll(self, ticket):
        info = SolveInfo()
        st = load().bmfp_server_poll(self.handle, ticket, ctypes.byref(info))
        if st == PENDING:
            return None
        if st not in (SUCCESS, ERROR_NOT_CONVERGED, ERROR_BREAKDOWN):
            check(st)
        self._keep.pop(ticket, None)
        return info.as_dict()

    def wait(self, ticket):
        info = SolveInfo()
        st = load().bmfp_server_wait(self.handle, ticket, ctypes.byref(info))
        if st not in (SUCCESS, ERROR_NOT_CONVERGED, ERROR_BREAKDOWN):
            check(st)
        self._keep.pop(ticket, None)
        return info.as_dict()

    def stats(self):
        s = ServerStats()
        check(load().bmfp_server_get_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            load().bmfp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
