"""libbmfp.so loads on a host without a GPU and exports every function that
include/bmfp.h declares; the host-only entry points behave."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import block_matrix_format_performance_gb300 as bm
from block_matrix_format_performance_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The reference's own result.json keys (gpu/gpu_matrix_multiplier.cu, main.cpp).
REFERENCE_NAMES = {
    bm.CSR_SCALAR: "GPU CSR",
    bm.CSR_VECTOR: "GPU CSR-Vector",
    bm.BCSR_ROW_THREAD: "GPU BCSR (row major, thread per row)",
    bm.BCSR_ROW_WARP: "GPU BCSR (row major, warp per row)",
    bm.BCSR_COL_THREAD: "GPU BCSR (column major, thread per row)",
    bm.BCSR_COL_THREAD_TEMPLATE: "GPU BCSR (column major, thread per row, template)",
    bm.BCSR_COL_COAL_X: "GPU BCSR (column major, thread per row, coal x)",
    bm.BCSR_COL_COAL_X_TEMPLATE: "GPU BCSR (column major, thread per row, coal x, template)",
    bm.BCSR_COL_BY_COL: "GPU BCSR (column major, column-by-column)",
    bm.BCSR_COL_BY_COL_FASTDIV: "GPU BCSR (column major, column-by-column, int fastdiv)",
    bm.BCSR_COL_BY_COL_PO2: "GPU BCSR (column major, column-by-column, int po2)",
    bm.BCSR_COL_BY_COL_TEMPLATE: "GPU BCSR (column major, column-by-column, template)",
    bm.BCSR_JIT: "jit",
    bm.CUSPARSE_ROW: "GPU BSR (cuSPARSE, row major)",
    bm.CUSPARSE_COL: "GPU BSR (cuSPARSE, column major)",
}


def test_every_header_function_is_exported(lib):
    declared = _capi.header_functions()
    assert len(declared) > 20
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    for f in declared:
        assert hasattr(lib, f)


def test_ctypes_signatures_cover_the_header(lib):
    declared = set(_capi.header_functions())
    assert declared <= set(_capi.SIGNATURES), sorted(declared - set(_capi.SIGNATURES))


def test_variant_names_are_the_reference_keys(lib):
    for v, name in REFERENCE_NAMES.items():
        assert bm.variant_name(v) == name
    assert bm.variant_name(bm.BCSR_NATIVE) == "GPU BCSR (GB300 native)"
    assert bm.variant_name(-1) is None and bm.variant_name(bm.VARIANT_COUNT) is None
    assert bm.variant_layout(bm.BCSR_COL_BY_COL) == 1 and bm.variant_layout(bm.BCSR_ROW_WARP) == 0
    assert bm.variant_is_csr(bm.CSR_VECTOR) == 1 and bm.variant_is_csr(bm.BCSR_NATIVE) == 0


def test_no_device_is_reported_cleanly_on_cpu_host(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("host has a GPU")
    assert bm.device_count() == 0


def test_invalid_arguments_fail_without_touching_a_device(lib):
    st = lib.bmfp_bcsr_spmv(7, bm.BCSR_NATIVE, 1, 1, 2, 1, None, None, None, None, None, None)
    assert st == bm.ERROR_INVALID_VALUE
    assert b"dtype" in lib.bmfp_last_error()
    st = lib.bmfp_bcsr_spmv(bm.R64F, bm.CSR_VECTOR, 1, 1, 2, 1, None, None, None, None, None, None)
    assert st == bm.ERROR_INVALID_VALUE
    st = lib.bmfp_bcsr_spmv(bm.R64F, bm.BCSR_NATIVE, 4, 4, 2, 8, None, None, None, None, None, None)
    assert st == bm.ERROR_INVALID_VALUE and b"null" in lib.bmfp_last_error()
    # zero rows is a valid no-op
    assert lib.bmfp_bcsr_spmv(bm.R64F, bm.BCSR_NATIVE, 0, 0, 2, 0, None, None, None, None, None, None) == 0


def test_native_lane_heuristic(lib):
    assert bm.native_default_lanes(np.float64, 2, 8.0) == 4
    assert bm.native_default_lanes(np.float64, 2, 5.0) == 2  # short rows: one lane per scalar row
    assert bm.native_default_lanes(np.float64, 2, 9.0) == 2
    assert bm.native_default_lanes(np.float64, 32, 8.0) == 64  # one lane per scalar row
    assert bm.native_default_lanes(np.float32, 2, 8.0) == 2
    for bs in (2, 4, 8, 16, 32):
        for dt in (np.float32, np.float64):
            g = bm.native_default_lanes(dt, bs, 8.0)
            v = 2 if dt == np.float64 else 4
            assert g == 64 or (g in (2, 4, 8, 16, 32) and g * v >= bs)


def test_oracle_is_not_linked_into_the_product(lib):
    out = subprocess.run(["nm", "-D", _capi.LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "orc_" not in out
    for dp, _, files in os.walk(os.path.join(ROOT, "block_matrix_format_performance_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                text = open(os.path.join(dp, f)).read()
                assert "oracle" not in text.lower().replace("the oracle", ""), f


def test_solver_option_defaults(lib):
    o = bm.solver_options()
    assert o.precision == bm.SOLVE_FP64 and o.tolerance == 1e-10
    assert o.inner_tolerance == 1e-4 and o.inner_max_iterations == 1000
    assert o.ctas_per_sm == 4 and o.inner_stall_iterations == 64
    assert bm.solver_options(inner_stall_iterations=0).inner_stall_iterations == 0
