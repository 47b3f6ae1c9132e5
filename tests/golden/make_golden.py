"""Regenerate the golden fixtures in this folder from the reference's own code.

Runs ``oracle/_ref/ref_golden`` (the reference headers compiled in place by
``make -C oracle ref``; needs the reference sources, so it runs only where
they are mounted) and packs its raw outputs into compressed ``.npz`` files:

  ndiag_<dtype>_n<rows>_b<blocks>_bs<bs>.npz
      gen_n_diag_bcsr -> BCSR arrays, transpose_blocks output, BCSR->CSR
      (common/matrix_converters.h:32-49, 88-117, 157-196)
  bridge_f64.npz
      golden_gate_bridge_2d<double,int,false> stiffness (BCSR bs=2), rhs, CSR
      (fem_2d/golden_gate_bridge.h:767-878)
  bridge.vtk, bridge_disp.vtk
      its write_vtk output, plain and with displacement ((i mod 7) - 3) / 1000
      (fem_2d/golden_gate_bridge.h:239-282)
  compare_results.json
      which vector pairs compare_results flags (common/measurement_class.h:58-87)
  measurement.json
      measurement_class averages (common/measurement_class.{h,cpp})
  ndiag_6x3_bs2.mtx
      csr_matrix_class::write_mm text (common/matrix_converters.h:119-144)

Usage:  python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ref_golden")

NDIAG_CASES = [
    # (dtype, n_rows, blocks_per_row, bs)
    ("f64", 50, 6, 1), ("f64", 50, 6, 2), ("f64", 40, 6, 3), ("f64", 40, 6, 4),
    ("f64", 30, 5, 5), ("f64", 24, 6, 8), ("f64", 12, 4, 16), ("f64", 8, 3, 32),
    ("f64", 7, 7, 2), ("f64", 9, 1, 4),
    ("f32", 50, 6, 2), ("f32", 24, 6, 8), ("f32", 8, 3, 32), ("f32", 1000, 6, 2),
]


def run(*args, cwd=None):
    return subprocess.run([REF_BIN, *map(str, args)], check=True, cwd=cwd,
                          capture_output=True, text=True).stdout


def read_case(prefix, dt):
    meta = open(prefix + ".meta").read().split()
    nbr, nbc, bs, nnzb, nnz = map(int, meta)
    fdt = np.float64 if dt == "f64" else np.float32
    out = {"n_block_rows": nbr, "n_block_cols": nbc, "bs": bs, "nnzb": nnzb, "nnz": nnz}
    for f, d in (("bcsr_row_ptr", np.int32), ("bcsr_cols", np.int32), ("bcsr_vals", fdt),
                 ("bcsr_vals_colmajor", fdt), ("csr_row_ptr", np.int32), ("csr_cols", np.int32),
                 ("csr_vals", fdt)):
        out[f] = np.fromfile(prefix + "." + f, dtype=d)
    return out


def main():
    if not os.path.exists(REF_BIN):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        for dt, n, b, bs in NDIAG_CASES:
            prefix = os.path.join(tmp, f"nd_{dt}_{n}_{b}_{bs}")
            run("ndiag", dt, n, b, bs, prefix)
            case = read_case(prefix, dt)
            np.savez_compressed(os.path.join(HERE, f"ndiag_{dt}_n{n}_b{b}_bs{bs}.npz"), **case)

        prefix = os.path.join(tmp, "bridge")
        run("bridge", prefix, cwd=tmp)  # the bridge also writes nodes/forces/elements into cwd
        case = read_case(prefix, "f64")
        case["rhs"] = np.fromfile(prefix + ".rhs", dtype=np.float64)
        np.savez_compressed(os.path.join(HERE, "bridge_f64.npz"), **case)
        for suffix in (".vtk", "_disp.vtk"):
            with open(prefix + suffix) as src, open(os.path.join(HERE, "bridge" + suffix), "w") as dst:
                dst.write(src.read())

        # compare_results around its 1e-9 threshold, both element types.
        rng = np.random.default_rng(7)
        cases = []
        for dt in ("f64", "f32"):
            fdt = np.float64 if dt == "f64" else np.float32
            for rel in (0.0, 1e-6, 3e-5, 6e-5, 1e-4, 1e-3):
                b = rng.uniform(-1, 1, 257).astype(fdt)
                a = (b * (1 + rel * rng.uniform(-1, 1, 257))).astype(fdt)
                fa, fb = os.path.join(tmp, "a.bin"), os.path.join(tmp, "b.bin")
                a.tofile(fa)
                b.tofile(fb)
                flag = run("compare", dt, a.size, fa, fb).strip()
                cases.append({"dtype": dt, "a": a.tolist(), "b": b.tolist(), "flagged": flag == "FLAGGED"})
        with open(os.path.join(HERE, "compare_results.json"), "w") as f:
            json.dump(cases, f)

        meas = []
        for seq in ([(0.5, 1e9, 2e9), (0.25, 1e9, 1e9)], [(1e-5, 3.5e6, 7e5)], [(2.0, 0.0, 0.0)] * 3):
            flat = [v for t in seq for v in t]
            e, bw, fl = map(float, run("measure", *flat).split())
            meas.append({"runs": seq, "elapsed": e, "bandwidth": bw, "throughput": fl})
        with open(os.path.join(HERE, "measurement.json"), "w") as f:
            json.dump(meas, f, indent=1)

        run("mm", os.path.join(tmp, "mm"))
        with open(os.path.join(tmp, "mm.mtx")) as src, open(os.path.join(HERE, "ndiag_6x3_bs2.mtx"), "w") as dst:
            dst.write(src.read())
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    sys.exit(main())
