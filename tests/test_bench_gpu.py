"""bench.py's secondary workloads end to end on the GPU, at small sizes: the
reference-compatible result.json run (main.cpp:383-398) and the JSON lines of
the solve / batch workloads."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

# Format strings every bs of the reference's results/result.json carries
# (main.cpp:146 keys them by measurement_class::get_format()).
REFERENCE_FORMATS = (
    "CPU CSR", "GPU CSR", "GPU CSR-Vector", "GPU BCSR (row major, thread per row)",
    "GPU BCSR (row major, warp per row)", "GPU BCSR (column major, thread per row)",
    "GPU BCSR (column major, thread per row, template)", "GPU BCSR (column major, thread per row, coal x)",
    "GPU BCSR (column major, thread per row, coal x, template)", "GPU BCSR (column major, column-by-column)",
    "GPU BCSR (column major, column-by-column, template)", "GPU BCSR (column major, column-by-column, int po2)",
    "GPU BCSR (column major, column-by-column, int fastdiv)", "GPU BSR (cuSPARSE, row major)",
    "GPU BSR (cuSPARSE, column major)")


def run_bench(*argv, timeout=900):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *argv], capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-3000:]
    return json.loads(p.stdout.strip().splitlines()[-1], parse_constant=_no_nan)  # strict JSON


def _no_nan(token):
    raise ValueError(f"{token} in the JSON line")


def test_ndiag_writes_reference_result_json(cuda, tmp_path):
    out = tmp_path / "result.json"
    line = run_bench("--workload", "ndiag", "--ndiag-rows", "3000", "--results-json", str(out))
    res = json.load(open(out))
    assert sorted(res, key=int) == ["2", "4", "8", "16", "32"]
    for bs, formats in res.items():
        for f in REFERENCE_FORMATS:
            assert f in formats, (bs, f)
        assert "GPU BCSR (GB300 native)" in formats
        assert all(t > 0 for t in formats.values())
        assert line["worst_compare_results"][bs] <= 1e-9
    assert line["results"] == res


def test_solve_workload_line(cuda):
    line = run_bench("--workload", "solve", "--grid", "40x10", "--repeats", "1")
    assert line["status"] == 0 and line["true_rel_residual"] < 1e-10


def test_batch_workload_line(cuda):
    line = run_bench("--workload", "batch", "--systems", "8", "--repeats", "1")
    assert line["systems"] == 8 and "fp64" in line and line["fp64"]["solves_per_s"] > 0
    assert "per_request_fp64" in line


def test_fma_peak_probe(cuda):
    import block_matrix_format_performance_gb300 as bm
    import numpy as np
    f64 = bm.measure_fma_peak(np.float64)
    f32 = bm.measure_fma_peak(np.float32)
    assert 50.0 < f64 < f32  # GFLOP/s; FP32 FMA is far faster than FP64 on GB300


def test_stream_read_floor(cuda):
    import torch
    import block_matrix_format_performance_gb300 as bm
    buf = torch.ones(1 << 20, dtype=torch.float32, device="cuda")
    bm.stream_read(buf)  # 4 MB, the whole buffer
    bm.stream_read(buf, 0)
    torch.cuda.synchronize()
    with pytest.raises(bm.BmfpError):  # not a multiple of 16 bytes
        bm.stream_read(buf, 24)
    with pytest.raises(bm.BmfpError):  # misaligned start
        bm.stream_read(buf[1:], 16)


def test_bridge_workload_line(cuda, tmp_path):
    out = tmp_path / "bridge.json"
    line = run_bench("--workload", "bridge", "--bridge-main-span", "1280", "--results-json", str(out))
    res = json.load(open(out))["2"]
    for f in REFERENCE_FORMATS:
        assert f in res, f
    assert line["spmv_seconds"] == res and line["worst_compare_results"] <= 1e-9
    assert line["block_rows"] > 1000 and line["solve"]["status"] == 0
    assert line["solve"]["recursive_rel_residual"] < 0.8
