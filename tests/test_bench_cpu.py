"""bench.py's reference arm on CPU: the JSON line the reference comparison
reads (the oracle's restatement of the reference CPU loop, timed on all host
threads), on a reduced selection so it runs in seconds."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _no_nan(token):
    raise ValueError(f"{token} in the JSON line")


def test_reference_arm_line(lib, orc):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--sizes", "2,4", "--dtypes", "f64"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1], parse_constant=_no_nan)  # strict JSON
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_only_rank0_prints(lib, orc):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--sizes", "2", "--dtypes", "f64"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert p.returncode == 0 and p.stdout.strip() == ""


def test_json_lines_are_strict():
    # a quantity not measured (NaN) or unbounded is written as null, never NaN
    sys.path.insert(0, ROOT)
    import bench
    line = bench.json_line({"e2e": {"value": float("nan"), "s": float("inf")}, "v": [1.5, float("-inf")], "k": 2})
    assert json.loads(line, parse_constant=_no_nan) == {"e2e": {"value": None, "s": None}, "v": [1.5, None], "k": 2}


def test_reference_arm_loads_no_product_code(orc):
    """The reference arm times the oracle's restatement of the reference CPU
    loop on matrices from the oracle's own generator: the product package
    (and its libbmfp.so) is never imported."""
    code = ("import sys, types; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--sizes', '2', '--dtypes', 'f32']; import bench; bench.main(); "
            "assert not any(m.startswith('block_matrix_format_performance_gb300') for m in sys.modules), "
            "sorted(m for m in sys.modules if 'block_matrix' in m)")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    assert json.loads(p.stdout.strip().splitlines()[-1])["impl"] == "reference"


def test_committed_traffic_names_the_lane_mapping():
    """The roofline's DRAM traffic comes from a committed ncu capture of the
    dominant case; it applies only to the lane mapping that capture ran."""
    sys.path.insert(0, ROOT)
    import bench
    t = bench.committed_traffic("bcsr_native_bs32_f64_lanes65")
    assert t is not None and 6.0e9 < t < 7.0e9
    assert bench.committed_traffic("bcsr_native_bs32_f64_lanes64") is None


def test_fifo_timeline_and_request_stream():
    """The FIFO baseline's timeline (done_k = max(done_k-1, arrival_k) +
    service_k) on a hand-checked case, and the seeded request stream:
    deterministic, Poisson arrivals at the stated rate, grids as the uneven
    batch plus the stated share of 1000x250 requests."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    t = bench.fifo_timeline([0.0, 0.5, 5.0], [1.0, 1.0, 2.0])
    # done: 1.0, 2.0 (waits for the first), 7.0 (idle until 5.0); latencies 1.0, 1.5, 2.0
    assert t["makespan_s"] == 7.0 and abs(t["solves_per_s"] - 3 / 7.0) < 0.01
    assert t["latency_p50_s"] == 1.5
    a1, g1 = bench.serve_stream(5000, 2000.0)
    a2, g2 = bench.serve_stream(5000, 2000.0)
    assert np.array_equal(a1, a2) and g1 == g2
    assert np.all(np.diff(a1) > 0) and abs(len(a1) / a1[-1] - 2000.0) < 100.0
    big = sum(g == (1000, 250) for g in g1)
    assert 200 < big < 300  # 5 % of 5000
    small = [g for g in g1 if g != (1000, 250)]
    assert all(20 <= nx <= 400 and ny == max(2, round(nx / 4)) for nx, ny in small)
