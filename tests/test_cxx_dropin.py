"""The C++ drop-in headers (include/bmfp/*.h) compiled like the reference's
own main.cpp would be: the same class and function names, linked against
libbmfp.so. Host-only use is checked against the golden vectors of the
reference's headers; the GPU program runs the reference's measurement flow
and solver call."""
import os
import subprocess

import numpy as np
import pytest

from block_matrix_format_performance_gb300 import build as B
from conftest import GOLDEN, ROOT, load_golden

CXX = os.environ.get("CXX", "g++")


def compile_cxx(src, out, tmp):
    pkg = os.path.dirname(B.LIB)
    cuda = B.cuda_home()
    cmd = [CXX, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include", "bmfp"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cxx", src), "-o", str(tmp / out),
           "-L", pkg, "-l:libbmfp.so", f"-Wl,-rpath,{pkg}", "-L", os.path.join(cuda, "lib64"), "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return str(tmp / out)


@pytest.fixture(scope="module")
def host_bin(lib, tmp_path_factory):
    tmp = tmp_path_factory.mktemp("cxx")
    return compile_cxx("host_dropin.cpp", "host_dropin", tmp)


@pytest.mark.parametrize("name", ["ndiag_f64_n50_b6_bs2.npz", "ndiag_f64_n40_b6_bs3.npz", "ndiag_f32_n24_b6_bs8.npz",
                                  "ndiag_f64_n8_b3_bs32.npz"])
def test_host_headers_match_reference_golden(host_bin, tmp_path, name):
    g = load_golden(name)
    dt = "f32" if g["bcsr_vals"].dtype == np.float32 else "f64"
    nbr = int(g["n_block_rows"])
    subprocess.run([host_bin, str(tmp_path), dt, str(nbr), str(int(g["nnzb"]) // nbr), str(int(g["bs"]))], check=True,
                   capture_output=True)
    for field in ("bcsr_row_ptr", "bcsr_cols", "bcsr_vals", "bcsr_vals_colmajor", "csr_row_ptr", "csr_cols", "csr_vals"):
        got = np.fromfile(tmp_path / field, dtype=g[field].dtype)
        assert np.array_equal(got.view(np.uint8), g[field].view(np.uint8)), field


def test_write_mm_is_byte_identical(host_bin, tmp_path):
    subprocess.run([host_bin, str(tmp_path), "mm"], check=True)
    assert open(tmp_path / "out.mtx").read() == open(os.path.join(GOLDEN, "ndiag_6x3_bs2.mtx")).read()


def test_golden_gate_bridge_class_matches_reference(host_bin, tmp_path):
    # golden_gate_bridge_2d<double, int, false> through the drop-in header:
    # matrix, load vector and write_vtk output as the reference's own class
    g = load_golden("bridge_f64.npz")
    subprocess.run([host_bin, str(tmp_path), "bridge"], check=True, capture_output=True)
    for field, ref in (("bcsr_row_ptr", g["bcsr_row_ptr"]), ("bcsr_cols", g["bcsr_cols"]),
                       ("bcsr_vals", g["bcsr_vals"]), ("rhs", g["rhs"])):
        got = np.fromfile(tmp_path / field, dtype=ref.dtype)
        assert np.array_equal(got.view(np.uint8), np.ascontiguousarray(ref).view(np.uint8)), field
    for name in ("bridge.vtk", "bridge_disp.vtk"):
        assert open(tmp_path / name).read() == open(os.path.join(GOLDEN, name)).read(), name


def test_measurement_class_matches_reference(host_bin, tmp_path):
    import json
    ref = json.load(open(os.path.join(GOLDEN, "measurement.json")))[0]
    out = subprocess.run([host_bin, str(tmp_path), "measure"], check=True, capture_output=True, text=True).stdout.split()
    assert [float(v) for v in out[:3]] == [ref["elapsed"], ref["bandwidth"], ref["throughput"]]
    assert out[3] == "m"


@pytest.mark.gpu
def test_reference_flow_on_gpu(lib, cuda, tmp_path):
    exe = compile_cxx("gpu_dropin.cpp", "gpu_dropin", tmp_path)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    assert "ERROR" not in p.stderr, p.stderr  # compare_results stayed quiet for every variant
    lines = p.stdout.splitlines()
    formats = {ln.split("\t")[0].split(" ", 2)[2] for ln in lines if not ln.startswith("solve")}
    for f in ("GPU CSR", "GPU CSR-Vector", "GPU BCSR (row major, thread per row)",
              "GPU BCSR (column major, thread per row, coal x)", "GPU BSR (cuSPARSE, row major)",
              "GPU BCSR (column major, column-by-column, template)", "GPU BCSR (GB300 native)"):
        assert f in formats, f
    # bs = 3: no power-of-two variant, like the reference's skip (gpu_matrix_multiplier.cu:1226)
    assert not any(ln.startswith("3 ") and "int po2" in ln for ln in lines)
    solves = [ln for ln in lines if ln.startswith("solve")]
    assert len(solves) == 3
    for ln in solves:
        kv = dict(t.split("=") for t in ln.split()[2:])
        eps = 1e-8 if "f64" in ln else 1e-4
        # the reference's stopping rule is the recursive residual
        assert float(kv["recursive"]) < eps, ln
        if "f64" in ln:
            assert float(kv["true"]) < 10 * eps, ln
        else:
            # FP32 BiCGStab on an elasticity operator drifts: the true
            # residual is reported, bounded only loosely
            assert np.isfinite(float(kv["true"])) and float(kv["true"]) < 1.0, ln
