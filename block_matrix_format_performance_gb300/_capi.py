"""ctypes declarations of libbmfp.so's C ABI (include/bmfp.h).

Loading fails loudly: there is no Python or CPU fallback for any device
entry point. Build the library with ``python -m block_matrix_format_performance_gb300.build``.
"""
from __future__ import annotations

import ctypes
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libbmfp.so")
HEADER = os.path.join(os.path.dirname(_PKG), "include", "bmfp.h")

c_int, c_int64, c_uint64, c_double, c_void_p, c_char_p = (
    ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p)
P = ctypes.POINTER

_LIB = None

# name -> (restype, argtypes)
SIGNATURES = {
    "bmfp_last_error": (c_char_p, []),
    "bmfp_version": (c_int, []),
    "bmfp_device_count": (c_int, []),
    "bmfp_spmv_variant_name": (c_char_p, [c_int]),
    "bmfp_spmv_variant_layout": (c_int, [c_int]),
    "bmfp_spmv_variant_is_csr": (c_int, [c_int]),
    "bmfp_csr_spmv": (c_int, [c_int, c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p]),
    "bmfp_bcsr_spmv": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int64, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_bcsr_spmv_native_ex": (c_int, [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_int, c_void_p]),
    "bmfp_bcsr_native_default_lanes": (c_int, [c_int, c_int, c_double]),
    "bmfp_mm_read_csr": (c_int, [ctypes.c_char_p, c_int, P(c_int), P(c_int), P(c_int64), c_void_p, c_void_p,
                                 c_void_p]),
    "bmfp_bcsr_spmv_colmajor": (c_int, [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
    "bmfp_matrix_set_lanes": (c_int, [c_void_p, c_int, c_void_p]),
    "bmfp_measure_fma_peak": (c_int, [c_int, P(c_double), c_void_p]),
    "bmfp_stream_read": (c_int, [c_void_p, ctypes.c_size_t, c_void_p]),
    "bmfp_bcsr_spmv_host": (c_int, [c_int, c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_int, c_void_p]),
    "bmfp_matrix_create_bcsr": (c_int, [P(c_void_p), c_int, c_int, c_int, c_int, c_int64, c_void_p,
                                        c_void_p, c_void_p, c_void_p]),
    "bmfp_matrix_create_csr": (c_int, [P(c_void_p), c_int, c_int, c_int, c_int64, c_void_p, c_void_p,
                                       c_void_p, c_void_p]),
    "bmfp_matrix_create_bcsr_device": (c_int, [P(c_void_p), c_int, c_int, c_int, c_int, c_int64,
                                               c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_matrix_convert": (c_int, [P(c_void_p), c_void_p, c_int, c_void_p]),
    "bmfp_matrix_destroy": (c_int, [c_void_p]),
    "bmfp_matrix_info": (c_int, [c_void_p, P(c_int), P(c_int), P(c_int), P(c_int), P(c_int64), P(c_int64)]),
    "bmfp_matrix_device_arrays": (c_int, [c_void_p, P(c_void_p), P(c_void_p), P(c_void_p)]),
    "bmfp_matrix_spmv": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_matrix_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, P(c_int)]),
    "bmfp_bcsr_to_csr": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "bmfp_csr_to_bcsr": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                 P(c_int64), c_void_p, c_void_p]),
    "bmfp_transpose_blocks": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "bmfp_gen_n_diag_bcsr": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "bmfp_gen_band_bcsr": (c_int, [c_int, c_int, c_int, c_int, c_int, c_uint64, c_void_p, P(c_int64),
                                   c_void_p, c_void_p]),
    "bmfp_gen_uniform_vector": (c_int, [c_int, c_int64, c_uint64, c_uint64, c_void_p]),
    "bmfp_gen_golden_gate_bridge": (c_int, [c_int, c_double, c_double, c_double, c_double, c_double, c_double,
                                            P(c_int), P(c_int64), c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_golden_gate_bridge_geometry": (c_int, [c_int, c_double, c_double, c_double, c_double, P(c_int), P(c_int),
                                                 P(c_int), c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_gen_q4_elasticity": (c_int, [c_int, c_int, c_int, c_double, c_double, c_void_p, P(c_int64),
                                       c_void_p, c_void_p, c_void_p]),
    "bmfp_bcsr_spmv_bytes": (c_int64, [c_int, c_int, c_int, c_int, c_int64]),
    "bmfp_solver_options_init": (None, [c_void_p]),
    "bmfp_solver_create": (c_int, [P(c_void_p), c_void_p, c_void_p, c_void_p]),
    "bmfp_solver_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_solver_destroy": (c_int, [c_void_p]),
    "bmfp_selftest_barrier_timeout": (c_int, [c_double, P(c_int), P(c_double), c_void_p]),
    "bmfp_batch_create": (c_int, [P(c_void_p), c_int, c_void_p, c_void_p, c_void_p]),
    "bmfp_batch_configure": (c_int, [c_void_p, c_int, c_int]),
    "bmfp_batch_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_int), P(c_int), c_void_p]),
    "bmfp_batch_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "bmfp_batch_destroy": (c_int, [c_void_p]),
    "bmfp_server_options_init": (None, [c_void_p]),
    "bmfp_server_create": (c_int, [P(c_void_p), c_void_p]),
    "bmfp_server_submit": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, P(c_uint64)]),
    "bmfp_server_poll": (c_int, [c_void_p, c_uint64, c_void_p]),
    "bmfp_server_wait": (c_int, [c_void_p, c_uint64, c_void_p]),
    "bmfp_server_get_stats": (c_int, [c_void_p, c_void_p]),
    "bmfp_server_destroy": (c_int, [c_void_p]),
    "bmfp_bicgstab_solve_noalloc": (c_int, [c_int, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p,
                                            c_void_p, c_void_p, c_double, c_int, c_int, P(c_int),
                                            P(c_double), c_void_p]),
    "bmfp_csr_spmv_bytes": (c_int64, [c_int, c_int, c_int, c_int64]),
}


class SolverOptions(ctypes.Structure):
    """struct bmfp_solver_options (include/bmfp.h)."""
    _fields_ = [("precision", c_int), ("preconditioner", c_int), ("tolerance", c_double),
                ("max_iterations", c_int), ("check_true_residual", c_int), ("inner_tolerance", c_double),
                ("inner_max_iterations", c_int), ("max_refinements", c_int), ("fallback_fp64", c_int),
                ("iterations_per_graph", c_int), ("ctas_per_sm", c_int), ("inner_stall_iterations", c_int),
                ("residual_replacement", c_int), ("launch_mode", c_int)]


class SolveInfo(ctypes.Structure):
    """struct bmfp_solve_info (include/bmfp.h)."""
    _fields_ = [("status", c_int), ("iterations", c_int), ("iterations_fp32", c_int), ("refinements", c_int),
                ("restarts", c_int), ("used_fp64_fallback", c_int), ("true_rel_residual", c_double),
                ("recursive_rel_residual", c_double), ("seconds", c_double), ("replacements", c_int),
                ("pad", c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class ServerOptions(ctypes.Structure):
    """struct bmfp_server_options (include/bmfp.h)."""
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_in_flight", c_int), ("max_batch", c_int),
                ("streams", c_int), ("cluster_size", c_int), ("threads_per_cta", c_int),
                ("wide_threshold_rows", c_int64), ("wide_lanes", c_int), ("solver", SolverOptions)]


class ServerStats(ctypes.Structure):
    """struct bmfp_server_stats (include/bmfp.h)."""
    _fields_ = [("submitted", c_uint64), ("completed", c_uint64), ("micro_batches", c_uint64),
                ("wide_solves", c_uint64), ("bytes_in_use", ctypes.c_size_t), ("peak_bytes", ctypes.c_size_t),
                ("in_flight", c_int), ("pending", c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BmfpError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"bmfp status {status}: {message}")
        self.status = status


def load(path: str | None = None):
    """Load libbmfp.so (once) and declare every signature."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m block_matrix_format_performance_gb300.build`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int):
    if status != 0:
        msg = load().bmfp_last_error()
        raise BmfpError(status, msg.decode() if msg else "")
    return status


def header_functions(header: str = HEADER):
    """Names of every function include/bmfp.h declares."""
    text = open(header).read()
    return sorted(set(re.findall(r"BMFP_API\s+[\w\s\*]+?\b(bmfp_\w+)\s*\(", text)))
