import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def lib():
    """libbmfp.so, built in-tree if missing or stale."""
    from block_matrix_format_performance_gb300 import build as B, _capi
    B.build()
    return _capi.load()


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")


def golden_cases(prefix):
    return sorted(f for f in os.listdir(GOLDEN) if f.startswith(prefix) and f.endswith(".npz"))


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def spmv_tolerance(orc, row_ptr, cols, vals, x, dtype):
    """Per-entry bound on |y_gpu - y_cpu|.

    float64: 1e-12 * sum_j |a_ij x_j| (the stated 1e-12 relative accuracy,
    scaled by |A||x| so that cancellation cannot make it vacuous).
    float32: 2 * n_i * 2^-24 * sum_j |a_ij x_j| with n_i the row's entry count:
    the worst-case rounding of two different summation orders (twice
    gamma_n), since GPU and CPU both round to float32 at every step.
    """
    scale = orc.abs_row_sums(row_ptr, cols, vals, x)
    if np.dtype(dtype) == np.float64:
        return 1e-12 * scale
    n_i = np.diff(np.asarray(row_ptr, dtype=np.int64)).astype(np.float64)
    return 2.0 * np.maximum(n_i, 1.0) * 2.0 ** -24 * scale
