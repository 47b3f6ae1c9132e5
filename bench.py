#!/usr/bin/env python
"""BCSR SpMV block-size sweep on GB300 — the benchmark line.

Workload (one "step"): y = A x once for each of 12 matrices — the seeded
random-band BCSR family with 100 000 block rows, 8 distinct block columns per
block row drawn from a +-64 band, block sizes 1, 2, 4, 8, 16, 32, in FP64 and
in FP32 (values and x uniform in [-1, 1)). Data are synthetic by
construction: the reference has no dataset, only generated matrices.

  value        algorithmic bytes of all 12 products / their summed device time
               (CUDA events around each product on the launching stream), GB/s.
               Bytes per product = values + 4-byte block columns + row offsets
               + x read once + y written once.
  L2           flushed before every product (write a 256 MB buffer, then read a
               512 MB one so no dirty line is written back inside the timed
               product); the flush is outside the events.
  e2e          the same bytes over the wall time of the user-facing call path
               with host buffers: bmfp_matrix_create_bcsr from pinned host
               arrays (allocation + upload), x upload, bmfp_matrix_spmv, y
               download, handle release — copies inside the timed region.
  roofline     the dominant product (largest share of device time) against
               MEASURED_PEAKS.json's HBM copy bandwidth.
  read floor   per product (per_case[*].read_floor_us): a plain streaming read
               of the same bytes after the same flush (bmfp_stream_read), the
               size-matched floor that launch ramp and DRAM latency set for
               the small products.
  cpu_baseline the oracle's restatement of the reference CPU loop
               (main.cpp:36-45, one thread) on the first rows of every matrix.

`--impl reference` times the reference's CPU path (the same loop, all host
threads) on a bounded sample of the same sweep and prints the same metric.

Multi-GPU: replicas only — every rank runs the whole sweep on its own GPU
(no collective on the data path); value sums the ranks' bytes over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NBR, BPR, HALF_BAND, SEED, X_STREAM = 100_000, 8, 64, 0, 2
BLOCK_SIZES = (1, 2, 4, 8, 16, 32)
DTYPES = ("f64", "f32")
METRIC = "SpMV GB/s vs HBM peak"
WORKLOAD = ("BCSR SpMV block-size sweep: 100000 block rows, 8 blocks/row drawn from a +-64 band, "
            "bs 1,2,4,8,16,32, FP64 and FP32, x uniform in [-1,1)")
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-csr-compare", action="store_true")
    ap.add_argument("--no-ref-variants", action="store_true",
                    help="skip timing the reference's own kernels on the sweep matrices")
    ap.add_argument("--no-solver", action="store_true", help="skip the batched-solve part of the line")
    ap.add_argument("--no-fem", action="store_true", help="skip the FEM solves (200x50, 2000x500) of the line")
    ap.add_argument("--no-serve", action="store_true", help="skip the served request stream of the line")
    ap.add_argument("--serve-requests", type=int, default=5000, help="line: requests of the served stream")
    ap.add_argument("--sustained-requests", type=int, default=2500,
                    help="line: requests of the sustained-rate stream (the first of the same stream)")
    ap.add_argument("--serve-precisions", default="mixed",
                    help="line: server precisions at the stated rate (the first also runs at the sustained rate)")
    ap.add_argument("--sustained-factor", type=float, default=0.7,
                    help="line: sustained rate as a fraction of the first server's throughput at the stated rate")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the autotuner's GB300 picks (built-in table, column owner at FP64 bs 16/32) "
                         "instead of timing candidates")
    ap.add_argument("--sizes", default=",".join(map(str, BLOCK_SIZES)))
    ap.add_argument("--dtypes", default=",".join(DTYPES))
    ap.add_argument("--n-block-rows", type=int, default=NBR,
                    help="block rows per matrix (smaller only for profiling captures)")
    ap.add_argument("--workload", choices=("spmv", "solve", "batch", "serve", "ndiag", "bridge", "precond"), default="spmv",
                    help="spmv: the block-size sweep line (default); solve: one Q4 elasticity solve; "
                         "batch: 256 uneven Q4 systems in one persistent launch; serve: Poisson request "
                         "stream through the server; ndiag: every variant on gen_n_diag_bcsr matrices, "
                         "written in the reference's result.json layout; bridge: the Golden Gate truss "
                         "through every format and main.cpp's Jacobi BiCGStab solve")
    ap.add_argument("--bridge-main-span", type=float, default=128000.0,
                    help="bridge: main span in metres (main.cpp:354 uses 128 km)")
    ap.add_argument("--results-json", default=None, help="ndiag: write {bs: {format: seconds}} here")
    ap.add_argument("--ndiag-rows", type=int, default=50_000, help="ndiag: block rows")
    ap.add_argument("--ndiag-dtype", default="f32", choices=("f32", "f64"))
    ap.add_argument("--systems", type=int, default=256, help="batch: number of systems")
    ap.add_argument("--batch-grid", default=None, help="batch: one NXxNY grid for every system (default: uneven)")
    ap.add_argument("--batch-config", default=None,
                    help="batch: CLUSTERxTHREADS for every precision instead of the autotuner's pick")
    ap.add_argument("--requests", type=int, default=1000, help="serve: number of requests")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: Poisson arrival rate (req/s)")
    ap.add_argument("--wide-lanes", type=int, default=None, help="serve: concurrent whole-GPU solves")
    ap.add_argument("--wide-threshold", type=int, default=None, help="serve: rows from which a request "
                                                                          "takes a whole-GPU lane")
    ap.add_argument("--no-baseline", action="store_true", help="serve: skip the FIFO per-request baseline")
    ap.add_argument("--large-fraction", type=float, default=0.05, help="serve: share of 1000x250 requests")
    ap.add_argument("--cluster-size", type=int, default=None, help="serve: CTAs per system team")
    ap.add_argument("--threads-per-cta", type=int, default=None, help="serve: threads per team CTA")
    ap.add_argument("--grid", default="200x50", help="solve: nodes nx x ny of the Q4 grid")
    ap.add_argument("--matrix", default="q4", choices=("q4", "shifted"),
                    help="solve: Q4 elasticity K (default) or the implicit-step operator K + shift * I")
    ap.add_argument("--shift", type=float, default=1e-3, help="solve: shift of --matrix shifted")
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp32", "mixed", "both"))
    ap.add_argument("--rhs", type=int, default=5, help="precond: right-hand sides (the load, then random loads)")
    ap.add_argument("--preconditioner", default="none", choices=("none", "jacobi", "block_jacobi"),
                    help="solve: right preconditioner of the single-system solver")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--max-iters", type=int, default=200000)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--ctas-per-sm", type=int, default=0,
                    help="solve / serve: persistent grid of the single-system solver (0 = default)")
    return ap.parse_args()


# Sweep cases where bmfp_matrix_autotune picks BMFP_LANES_COL_OWNER on GB300.
COLUMN_OWNER_CASES = {("f64", 16): 65, ("f64", 32): 65}


def np_dt(tag):
    return np.float64 if tag == "f64" else np.float32


def case_bytes(bs, tag, nnzb, nbr=NBR):
    S = 8 if tag == "f64" else 4
    return nnzb * bs * bs * S + nnzb * 4 + (nbr + 1) * 4 + 2 * nbr * bs * S


def json_line(obj):
    """One strict JSON line: non-finite floats (a quantity not measured or not
    evaluated) become null, since NaN and Infinity are not JSON."""
    def clean(o):
        if isinstance(o, float) and not math.isfinite(o):
            return None
        if isinstance(o, dict):
            return {k: clean(v) for k, v in o.items()}
        if isinstance(o, (list, tuple)):
            return [clean(v) for v in o]
        return o
    return json.dumps(clean(obj), allow_nan=False)


def max_over_ranks(value, dist, device):
    """Largest per-rank value (the slowest replica's time); the value itself on
    a single process. Replicas exchange only this scalar — no data-path
    collective."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(total_bytes_per_rank, world, t_max_s):
    """Whole-job GB/s: every rank's bytes over the slowest rank's time."""
    return world * total_bytes_per_rank / t_max_s / 1e9


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi SM clock and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [s.strip() for s in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                mhz.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(mhz)}


# ---------------------------------------------------------------- workload

def build_cases(bm, sizes, dtypes, nbr):
    cases = []
    for tag in dtypes:
        for bs in sizes:
            rp, c, v = bm.gen_band_bcsr(nbr, BPR, HALF_BAND, bs, SEED, np_dt(tag))
            x = bm.gen_uniform_vector(nbr * bs, SEED, X_STREAM, np_dt(tag))
            case = {"bs": bs, "tag": tag, "rp": rp, "c": c, "v": v, "x": x, "nnzb": int(c.size),
                    "bytes": case_bytes(bs, tag, int(c.size), nbr)}
            cases.append(case)
    return cases


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def read_floor_us(byte_counts, flush, stream, reps=20):
    """Device time of a plain streaming read of each byte count (bmfp_stream_read),
    timed exactly like the products: L2 flushed, then CUDA events around one
    launch. The size-matched floor of a small product: launch ramp, first DRAM
    round trips and tail cost every kernel a few microseconds."""
    import torch
    import block_matrix_format_performance_gb300 as bm
    buf = torch.empty((max(byte_counts) + 15) // 16 * 4, dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = []
    for nb in byte_counts:
        nb16 = (nb + 15) // 16 * 16
        total = 0.0
        for r in range(reps + 2):
            flush()
            e0.record(stream)
            bm.stream_read(buf, nb16, stream=stream)
            e1.record(stream)
            e1.synchronize()
            if r >= 2:
                total += e0.elapsed_time(e1)
        out.append(total / reps * 1e3)
    del buf
    return out


def committed_traffic(kernel_key):
    """dram bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.md line `traffic <key>: <bytes>`), or None. The key
    names the case and the lane mapping the capture ran (`..._lanes<L>`): a
    run that picks another mapping finds no line and reports null rather than
    another kernel's bytes."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    pat = re.compile(r"traffic\s+" + re.escape(kernel_key) + r"\s*:\s*([0-9.eE+]+)")
    for f in sorted(os.listdir(pdir)):
        if f.endswith((".md", ".txt")):
            m = pat.search(open(os.path.join(pdir, f)).read())
            if m:
                return float(m.group(1))
    return None


def run_ours(args):
    import torch

    import block_matrix_format_performance_gb300 as bm
    from block_matrix_format_performance_gb300 import build as B

    rank, world, local = dist_env()
    B.build()
    bm.load()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    sizes = [int(s) for s in args.sizes.split(",")]
    dtypes = args.dtypes.split(",")
    t0 = time.time()
    nbr = args.n_block_rows
    cases = build_cases(bm, sizes, dtypes, nbr)
    gen_s = time.time() - t0

    stream = torch.cuda.current_stream()
    for cs in cases:
        cs["m"] = bm.Matrix.from_bcsr(cs["rp"], cs["c"], cs["v"], cs["bs"])
        cs["dx"] = torch.from_numpy(cs["x"]).cuda()
        cs["dy"] = torch.empty_like(cs["dx"])
        # the library's autotuner times every valid lane count on this matrix
        if args.no_autotune:
            # the autotuner's GB300 picks that the library's built-in table
            # cannot make (the column owner needs the handle's column-major copy)
            cs["lanes"] = COLUMN_OWNER_CASES.get((cs["tag"], cs["bs"]), 0)
            if cs["lanes"]:
                cs["m"].set_lanes(cs["lanes"])
        else:
            cs["lanes"] = cs["m"].autotune(cs["dx"], cs["dy"])
    flush_w = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB
    flush_r = torch.ones(128 << 20, dtype=torch.float32, device="cuda")  # 512 MB

    def flush():
        flush_w.zero_()
        flush_r.sum()

    n = len(cases)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(n)]
    for _ in range(args.warmup):
        for cs in cases:
            flush()
            cs["m"].spmv(cs["dx"], cs["dy"])
    torch.cuda.synchronize()

    per_case_ms = [0.0] * n
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            for i, cs in enumerate(cases):
                flush()
                ev[i][0].record(stream)
                cs["m"].spmv(cs["dx"], cs["dy"])
                ev[i][1].record(stream)
            torch.cuda.synchronize()  # events of this step are complete
            for i in range(n):
                per_case_ms[i] += ev[i][0].elapsed_time(ev[i][1])
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if dist:
        dist.barrier()

    step_ms = sum(per_case_ms) / args.steps
    total_bytes = sum(cs["bytes"] for cs in cases)
    t_max = max_over_ranks(step_ms, dist, "cuda")
    value = replica_value(total_bytes, world, t_max * 1e-3)

    # The second roofline of FP64 products: GB300's FP64 FMA rate, measured
    # here (one FMA per value, so at most bytes / (2 nnzb bs^2 / rate)).
    fp64_gflops = bm.measure_fma_peak(np.float64)
    read_us = read_floor_us([cs["bytes"] for cs in cases], flush, stream)
    per_case = {}
    for i, cs in enumerate(cases):
        ms = per_case_ms[i] / args.steps
        gbs = cs["bytes"] / (ms * 1e-3) / 1e9
        per_case[f"bs{cs['bs']}_{cs['tag']}"] = {"gbs": round(gbs, 1), "us": round(ms * 1e3, 2),
                                                  "mb": round(cs["bytes"] / 1e6, 1), "lanes": cs["lanes"],
                                                  "read_floor_us": round(read_us[i], 2),
                                                  "of_read_floor": round(read_us[i] / (ms * 1e3), 3)}
        if cs["tag"] == "f64":
            bound = cs["bytes"] / (2.0 * cs["nnzb"] * cs["bs"] ** 2 / (fp64_gflops * 1e9)) / 1e9
            per_case[f"bs{cs['bs']}_{cs['tag']}"]["of_min_hbm_fp64_bound"] = round(gbs / min(bound, peaks()[0]), 3)
    dom = max(range(n), key=lambda i: per_case_ms[i])
    dcs = cases[dom]
    dom_ms = per_case_ms[dom] / args.steps
    hbm, peak_kind = peaks()
    achieved = dcs["bytes"] / (dom_ms * 1e-3) / 1e9
    dom_key = f"bcsr_native_bs{dcs['bs']}_{dcs['tag']}_lanes{dcs['lanes']}"
    traffic = committed_traffic(dom_key)
    fp64_bound = None
    if dcs["tag"] == "f64":
        flops = 2.0 * dcs["nnzb"] * dcs["bs"] ** 2
        bound_gbs = dcs["bytes"] / (flops / (fp64_gflops * 1e9)) / 1e9
        fp64_bound = {"fp64_fma_gflops_measured": round(fp64_gflops, 1), "bound_gbs": round(bound_gbs, 1),
                      "frac": round(achieved / bound_gbs, 4),
                      "binding": "fp64_pipe" if bound_gbs < hbm else "hbm"}

    # CSR warp-per-row ("GPU CSR-Vector") on the same matrices, for comparison.
    csr_cmp = {}
    if not args.no_csr_compare:
        for cs in cases:
            crp, cc, cv = bm.bcsr_to_csr(cs["rp"], cs["c"], cs["v"], cs["bs"])
            d_rp, d_c, d_v = (torch.from_numpy(a).cuda() for a in (crp, cc, cv))
            cbytes = bm.csr_spmv_bytes(np_dt(cs["tag"]), nbr * cs["bs"], nbr * cs["bs"], cc.size)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps, tot = 5, 0.0
            for r in range(reps + 1):
                flush()
                e0.record(stream)
                bm.csr_spmv(bm.CSR_VECTOR, d_rp, d_c, d_v, cs["dx"], cs["dy"])
                e1.record(stream)
                torch.cuda.synchronize()
                if r:
                    tot += e0.elapsed_time(e1)
            ms = tot / reps
            csr_cmp[f"bs{cs['bs']}_{cs['tag']}"] = {
                "csr_vector_gbs": round(cbytes / (ms * 1e-3) / 1e9, 1),
                "csr_vector_us": round(ms * 1e3, 2),
                "native_speedup": round(ms / (per_case_ms[cases.index(cs)] / args.steps), 2)}
            del d_rp, d_c, d_v

    # The reference's own kernels (restated one per format string, the same
    # thread mappings) on the same matrices: row-major thread / warp per row,
    # column-major thread per row (template), column-by-column (template) and
    # cuSPARSE bsrmv. bs 1 is CSR, covered above.
    ref_cmp = {}
    if not args.no_ref_variants:
        ref_variants = [bm.BCSR_ROW_THREAD, bm.BCSR_ROW_WARP, bm.BCSR_COL_THREAD_TEMPLATE,
                        bm.BCSR_COL_BY_COL_TEMPLATE, bm.CUSPARSE_ROW]
        for cs in cases:
            if cs["bs"] == 1:
                continue
            d_rp, d_c, d_v = (torch.from_numpy(a).cuda() for a in (cs["rp"], cs["c"], cs["v"]))
            d_vt = None
            native_ms = per_case_ms[cases.index(cs)] / args.steps
            res = {}
            for var in ref_variants:
                if bm.variant_layout(var) == 1 and d_vt is None:
                    d_vt = torch.from_numpy(bm.transpose_blocks(cs["rp"], cs["v"], cs["bs"])).cuda()
                vals = d_vt if bm.variant_layout(var) == 1 else d_v
                try:
                    bm.bcsr_spmv(var, d_rp, d_c, vals, cs["dx"], cs["dy"], cs["bs"])
                except bm.BmfpError as e:
                    if e.status == bm.ERROR_NOT_SUPPORTED:
                        continue
                    raise
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                reps, tot = 3, 0.0
                for r in range(reps + 1):
                    flush()
                    e0.record(stream)
                    bm.bcsr_spmv(var, d_rp, d_c, vals, cs["dx"], cs["dy"], cs["bs"])
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if r:
                        tot += e0.elapsed_time(e1)
                res[bm.variant_name(var)] = round(cs["bytes"] / (tot / reps * 1e-3) / 1e9, 1)
            best = max(res, key=res.get)
            ref_cmp[f"bs{cs['bs']}_{cs['tag']}"] = {
                "best_reference_format": best, "best_reference_gbs": res[best],
                "native_speedup": round(cs["bytes"] / (native_ms * 1e-3) / 1e9 / res[best], 2), "gbs": res}
            del d_rp, d_c, d_v, d_vt
            torch.cuda.empty_cache()

    # End to end through the C ABI with host buffers: bmfp_bcsr_spmv_host
    # takes the pinned host arrays, uploads them in chunks overlapped with the
    # product and returns y in host memory, so every step moves the whole
    # matrix and x across the host link and y back.
    pinned = []
    for cs in cases:
        pinned.append(tuple(torch.from_numpy(a).pin_memory() for a in (cs["rp"], cs["c"], cs["v"], cs["x"])))
    h_y = [torch.empty(cs["x"].shape, dtype=torch.float64 if cs["tag"] == "f64" else torch.float32).pin_memory()
           for cs in cases]
    for cs in cases:
        cs["m"].close()
    h2d = sum(sum(t.numel() * t.element_size() for t in p) for p in pinned)
    d2h = sum(t.numel() * t.element_size() for t in h_y)

    def e2e_step():
        for cs, p, hy in zip(cases, pinned, h_y):
            bm.bcsr_spmv_host(p[0].numpy(), p[1].numpy(), p[2].numpy(), p[3].numpy(), cs["bs"], y=hy.numpy())

    e2e_s = float("nan")
    if args.e2e_steps > 0:
        e2e_step()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = (time.perf_counter() - e0) / args.e2e_steps
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    e2e_value = replica_value(total_bytes, world, e2e_s)

    del pinned, h_y
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sizes, dtypes, nbr=nbr)

    # Solver side of the metric: the uneven batch of elasticity systems at
    # 1e-10, batched FP64 and mixed against the plain FP64 per-request solver.
    solves = None
    if not args.no_solver:
        for cs in cases:
            cs.pop("m", None)
        torch.cuda.empty_cache()
        solves = measure_batch(["fp64", "mixed"], 1e-10, 100000, 2)
        solves_shifted = measure_batch(["fp64", "mixed"], 1e-10, 100000, 2, shift=1e-3)
    # The FEM workloads of configs 0 and 2, the live cost of one solver
    # iteration against its floors, and the served request stream.
    fem = None
    single = rank == 0 and world == 1  # the FEM and serving legs are one-GPU workloads
    if single and not args.no_fem:
        t0 = time.perf_counter()
        fem = {"q4_200x50": fem_small(flush, stream),
               "iteration_roofline": [iteration_roofline(g, hbm, fp64_gflops) for g in ((1000, 250), (2000, 500))],
               "q4_2000x500": fem_large(),
               "preconditioners": precond_compare(((1000, 250),), n_rhs=3)}
        fem["wall_s"] = round(time.perf_counter() - t0, 1)
    serve = None
    if single and not args.no_serve:
        t0 = time.perf_counter()
        serve = serve_suite(args.serve_requests, args.rate, args.serve_precisions.split(","), args.sustained_factor,
                            sustained_requests=args.sustained_requests)
        serve["wall_s"] = round(time.perf_counter() - t0, 1)

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_max, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "+".join(dtypes), "data": "synthetic (seeded generator; the reference has no dataset)",
        "config": {
            "workload": WORKLOAD if nbr == NBR else WORKLOAD.replace("100000", str(nbr)), "n_block_rows": nbr, "blocks_per_row": BPR, "half_band": HALF_BAND,
            "block_sizes": sizes, "seed": SEED, "parallelism": f"replicas x{world} (no collective)",
            "l2": "flushed before every product (256 MB write + 512 MB read), outside the timed events",
            "kernel": "GPU BCSR (GB300 native)", "per_case": per_case, "csr_warp_per_row": csr_cmp,
            "reference_variants": ref_cmp,
            "wall_s_timed_region": round(wall, 3), "generate_s": round(gen_s, 1),
        },
        "roofline": {"bound": "hbm", "kernel": dom_key, "achieved": round(achieved, 1), "peak": hbm,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s", "unit": "GB/s", "frac": round(achieved / hbm, 4),
                     "traffic": traffic, "algorithmic_bytes": dcs["bytes"], "fp64_pipe": fp64_bound},
        # not measured (--e2e-steps 0): null rather than NaN, which is not JSON
        "e2e": {"value": round(e2e_value, 2) if e2e_value == e2e_value else None, "unit": "GB/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "s_per_step": round(e2e_s, 4) if e2e_s == e2e_s else None},
        "gpu_launches": args.steps * n,
        "clocks": clocks.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if solves is not None:
        line["solves"] = {"workload": "256 uneven Q4 plane-stress systems, nx log-uniform in [20,400], ny = nx/4, "
                                      "bs 2, 1e-10 true relative residual", **solves}
        line["solves_implicit_step"] = {"workload": "the same 256 grids with K + 1e-3 I (implicit time step, unit "
                                                    "lumped mass): FP32 inner solves converge", **solves_shifted}
    if fem is not None:
        line["fem"] = fem
    if serve is not None:
        line["serve"] = serve
    if rank == 0:
        print(json_line(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------------------- CPU sides

# Written before every CPU product, outside the timing: more than twice the
# largest last-level cache of the hosts this runs on (Grace: 114 MB), so
# every product streams its matrix from DRAM, like the L2-flushed GPU side.
CPU_FLUSH_BYTES = 256 << 20


class CpuFlush:
    """Evicts the host's last-level cache by writing a buffer larger than it."""

    def __init__(self, nbytes=CPU_FLUSH_BYTES):
        self.buf = np.zeros(nbytes // 8, np.float64)
        self.k = 0.0

    def __call__(self):
        self.k += 1.0
        self.buf.fill(self.k)


def cpu_sweep(sizes, dtypes, nbr, threads, steps, warmup):
    """The reference CPU loop (main.cpp:36-45, restated in oracle.c) over the
    FULL sweep matrices as CSR, generated by the oracle's C restatement of the
    band generator (no product code), one matrix at a time: `warmup` untimed
    and `steps` timed products each, the host LLC flushed before every
    product (outside the timing). Bytes are the workload's algorithmic bytes
    (the BCSR formula, as on the GPU side). Returns (bytes per step, seconds
    per step, {case: GB/s})."""
    from oracle import oracle as orc
    orc.build()
    flush = CpuFlush()
    gen_threads = os.cpu_count() or 1
    tot_b, tot_s, per = 0, 0.0, {}
    for tag in dtypes:
        for bs in sizes:
            crp, cc, cv = orc.gen_band_c(nbr, BPR, HALF_BAND, bs, SEED, np_dt(tag), csr=True, threads=gen_threads)
            x = orc.gen_uniform_vector_c(nbr * bs, SEED, X_STREAM, np_dt(tag))
            y = np.zeros_like(x)
            nb = case_bytes(bs, tag, cv.size // (bs * bs), nbr)
            for _ in range(warmup):
                flush()
                orc.csr_spmv(crp, cc, cv, x, threads=threads, out=y)
            t = 0.0
            for _ in range(steps):
                flush()
                t0 = time.perf_counter()
                orc.csr_spmv(crp, cc, cv, x, threads=threads, out=y)
                t += time.perf_counter() - t0
            per[f"bs{bs}_{tag}"] = round(nb * steps / t / 1e9, 2)
            tot_b += nb
            tot_s += t / steps
            del crp, cc, cv
    return tot_b, tot_s, per


def cpu_baseline(sizes, dtypes, nbr=NBR, steps=2):
    """Oracle restatement of main.cpp:36-45 on one core (as the reference
    times it) over the full sweep."""
    b, sec, per = cpu_sweep(sizes, dtypes, nbr, 1, steps, 0)
    return {"value": round(b / sec / 1e9, 2), "unit": "GB/s", "cores": 1, "kind": "port",
            "sample": f"the full {nbr}-block-row sweep matrices as CSR ({len(sizes) * len(dtypes)} cases), {steps} "
                      "products each, the host LLC flushed (256 MB write) before every product; the reference "
                      "CPU loop main.cpp:36-45 restated in C (oracle/oracle.c, -O2, one thread); inputs from the "
                      "oracle's C band generator", "per_case_gbs": per}


def cpu_solve(grid, threads, max_iterations=100000, tol=1e-10):
    """The reference BiCGStab recurrences (gpu/bicgstab.cu:426-513, restated
    in oracle.c, last iterate returned) on the host: FP64, no
    preconditioner, on `threads` host threads (1 = orc_bicgstab_f64, the
    reference's single-threaded form). Returns the iterations, seconds and
    the true relative residual."""
    import block_matrix_format_performance_gb300 as bm
    from oracle import oracle as orc
    nx, ny = grid
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)  # host-side generator (the workload's input)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    del rp, c, v
    t0 = time.perf_counter()
    if threads == 1:
        x, st, it, rel = orc.bicgstab(crp, cc, cv, rhs, tol, max_iterations)
    else:
        x, st, it, rel = orc.bicgstab_mt(crp, cc, cv, rhs, tol, max_iterations, threads)
    sec = time.perf_counter() - t0
    y = orc.csr_spmv(crp, cc, cv, x, threads=max(1, threads))
    true_rel = float(np.linalg.norm(rhs - y) / np.linalg.norm(rhs))
    return {"threads": threads, "iterations": it, "seconds": round(sec, 4), "s_per_iteration": sec / max(it, 1),
            "status": st, "recursive_rel": rel, "true_rel": true_rel}


def run_reference(args):
    """The reference's CPU path on the host cores: the CSR loop of
    main.cpp:36-45 (restated in oracle.c: the reference's main.cpp needs the
    absent fmt and cuda_jit submodules) on all host threads over the full
    sweep matrices, generated by the oracle (no product code is imported)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sizes = [int(s) for s in args.sizes.split(",")]
    dtypes = args.dtypes.split(",")
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    b, sec, per = cpu_sweep(sizes, dtypes, NBR, threads, steps, args.warmup)
    wall = time.perf_counter() - t0
    value = b / sec / 1e9
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "+".join(dtypes), "data": "synthetic (seeded generator)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "block_sizes": sizes, "n_block_rows": NBR,
                   "llc": "flushed before every product (256 MB write), outside the timing", "wall_s": round(wall, 1)},
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"the full {NBR}-block-row sweep matrices as CSR, {steps} products each after "
                                   f"{args.warmup} untimed; the reference CPU loop main.cpp:36-45 restated in C "
                                   f"(oracle/oracle.c), rows split over {threads} threads; the reference's main.cpp "
                                   "needs the absent fmt and cuda_jit submodules, so it is not built",
                         "per_case_gbs": per},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json_line(line), flush=True)


def run_solve(args):
    """Q4 plane-stress solves (the FEM workloads), timed end to end on the
    device: solves/s, iterations, true residual and bytes per iteration.
    --precision both runs plain FP64 and FP32-inner / FP64-refined on the same
    system and reports the mixed solution's error against the FP64 one."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from block_matrix_format_performance_gb300 import build as B
    B.build()
    nx, ny = (int(t) for t in args.grid.lower().split("x"))
    if args.matrix == "shifted":
        rp, c, v, rhs = shifted_q4(nx, ny, args.shift)
    else:
        rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    d_b = torch.from_numpy(rhs).cuda()
    n = 2 * nx * ny
    out, xs = {}, {}
    for prec in (("fp64", "mixed") if args.precision == "both" else (args.precision,)):
        kw = {"ctas_per_sm": args.ctas_per_sm} if args.ctas_per_sm else {}
        s = bm.Solver(A, prec, tol=args.tol, max_iters=args.max_iters, preconditioner=args.preconditioner, **kw)
        d_x = torch.empty_like(d_b)
        infos = [s.solve(d_b, d_x) for _ in range(max(1, args.repeats))]
        s.close()
        best = min(infos, key=lambda i: i["seconds"])
        xs[prec] = d_x
        spmv_b = bm.bcsr_spmv_bytes(np.float64 if prec == "fp64" else np.float32, nx * ny, nx * ny, 2, int(c.size))
        per_iter = 2 * spmv_b + 17 * n * (8 if prec == "fp64" else 4)
        it = max(best["iterations"], 1)
        out[prec] = {"solves_per_s": round(1.0 / best["seconds"], 3), "seconds": round(best["seconds"], 4),
                     "us_per_iteration": round(best["seconds"] / it * 1e6, 2), "bytes_per_iteration": int(per_iter),
                     "gbs_per_iteration": round(per_iter / (best["seconds"] / it) / 1e9, 1), **best}
    line = {"workload": "solve", "matrix": args.matrix if args.matrix == "q4" else f"q4+{args.shift:g}I",
            "grid": [nx, ny], "dofs": n, "nnzb": int(c.size), "tol": args.tol}
    if len(out) == 1:
        line.update(precision=args.precision, **out[args.precision])
    else:
        line.update(out)
        ref = xs["fp64"].double()
        line["mixed_error_vs_fp64"] = float(torch.linalg.norm(xs["mixed"].double() - ref) / torch.linalg.norm(ref))
    print(json_line(line), flush=True)
    A.close()


def shifted_q4(nx, ny, shift):
    """The Q4 elasticity operator of an implicit time step, K + shift * I
    (unit lumped mass, shift = 1 / dt^2): on the 200x50 grid shift 1e-3 gives
    cond ~ 4e3 instead of K's 3e6, within reach of FP32 inner solves
    (u32 * cond ~ 3e-4), so it shows what mixed precision buys on GB300 where
    it can work."""
    import block_matrix_format_performance_gb300 as bm
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    v = v.reshape(-1, 2, 2).copy()
    rows = np.repeat(np.arange(nx * ny), np.diff(rp))
    v[c == rows] += shift * np.eye(2)
    return rp, c, v.reshape(-1), rhs


def batch_grids(n_systems, seed=0):
    """nx log-uniform in [20, 400] (seeded), ny = nx / 4: the uneven-batch workload."""
    rng = np.random.default_rng(seed)
    nxs = np.round(np.exp(rng.uniform(np.log(20), np.log(400), n_systems))).astype(int)
    return [(int(nx), max(2, int(round(nx / 4)))) for nx in nxs]


def fp64_floor(rp, c, v, bs, x, b):
    """u ||A| |x|| / ||b||, u = 2^-53: the rounding floor of b - A x evaluated
    in FP64 for this x (the residual of the correctly rounded solution is of
    this size too), so a system whose floor exceeds the tolerance cannot be
    expected to meet it in FP64."""
    import scipy.sparse as sp
    n = (len(rp) - 1) * bs
    A = sp.bsr_matrix((np.abs(np.asarray(v, np.float64)).reshape(-1, bs, bs), c, rp), shape=(n, n))
    return float(2.0 ** -53 * np.linalg.norm(A @ np.abs(x)) / np.linalg.norm(b))


def measure_batch(precisions, tol, max_iters, repeats, n_systems=256, per_request=True, grid=None, shift=None,
                  config=None):
    """The uneven batch (nx log-uniform in [20, 400], ny = nx / 4, seeded): each
    precision solved by one persistent, graph-captured launch, and the plain
    FP64 per-request solver run system after system on the same GPU (its
    solver objects built before the timed loop, their construction reported
    as setup_s). Each system's FP64 rounding floor (fp64_floor) is reported
    beside its true residual where it missed the tolerance."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    grids = batch_grids(n_systems) if grid is None else [grid] * n_systems
    mats, rhs, host = [], [], []
    for nx, ny in grids:
        rp, c, v, b = shifted_q4(nx, ny, shift) if shift else bm.gen_q4_elasticity(nx, ny)
        mats.append(bm.Matrix.from_bcsr(rp, c, v, 2))
        rhs.append(b)
        host.append((rp, c, v))
    d_b = [torch.from_numpy(b).cuda() for b in rhs]
    d_x = [torch.empty_like(b) for b in d_b]
    out = {"systems": len(grids), "dofs_total": int(sum(2 * a * b for a, b in grids)), "tol": tol}
    floors = {}

    def floor_of(k, x):
        if k not in floors:
            floors[k] = fp64_floor(*host[k], 2, x, rhs[k])
        return floors[k]

    for prec in precisions:
        batch = bm.Batch(mats, prec, tol=tol, max_iters=max_iters)
        t0 = time.perf_counter()
        if config:
            cluster, threads = config
            batch.configure(cluster, threads)
        else:
            cluster, threads = batch.autotune(d_b, d_x, probe_iterations=1024)
        tune_s = time.perf_counter() - t0
        batch.solve(d_b, d_x)
        times, infos = [], None
        for _ in range(max(1, repeats)):
            t0 = time.perf_counter()
            infos = batch.solve(d_b, d_x)
            times.append(time.perf_counter() - t0)
        batch.close()
        batch_s = min(times)
        missed = []
        for k, i in enumerate(infos):
            if i["status"] != 0:
                fl = floor_of(k, d_x[k].cpu().numpy())
                missed.append({"grid": grids[k], "true_rel": i["true_rel_residual"], "fp64_floor": fl})
        out[prec] = {
            "cluster": cluster, "threads_per_cta": threads, "autotune_s": round(tune_s, 3),
            "batch_s": round(batch_s, 4), "solves_per_s": round(len(grids) / batch_s, 2),
            "converged": sum(i["status"] == 0 for i in infos),
            "worst_true_rel": max(i["true_rel_residual"] for i in infos),
            "iterations": sum(i["iterations"] for i in infos),
            "iterations_fp32": sum(i["iterations_fp32"] for i in infos),
            "fp64_fallbacks": sum(i["used_fp64_fallback"] for i in infos),
            "replacements": sum(i["replacements"] for i in infos),
            "not_converged": missed[:16],
            "not_converged_below_floor": sum(m["fp64_floor"] < tol for m in missed)}
    if per_request:
        t0 = time.perf_counter()
        solvers = [bm.Solver(m, "fp64", tol=tol, max_iters=max_iters) for m in mats]
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        seq = []
        t0 = time.perf_counter()
        for sv, b, x in zip(solvers, d_b, d_x):
            seq.append(sv.solve(b, x))
        dt = time.perf_counter() - t0
        for sv in solvers:
            sv.close()
        out["per_request_fp64"] = {"seconds": round(dt, 4), "solves_per_s": round(len(grids) / dt, 2),
                                   "setup_s": round(setup_s, 3),
                                   "converged": sum(i["status"] == 0 for i in seq),
                                   "iterations": sum(i["iterations"] for i in seq)}
    if grid is None and shift is None:
        # every system's floor, from its last FP64 solution in d_x
        xs = [x.cpu().numpy() for x in d_x]
        fl = [floor_of(k, xs[k]) for k in range(len(grids))]
        out["fp64_floor_above_tol"] = sum(f > tol for f in fl)
        out["fp64_floor_max"] = max(fl)
    for m in mats:
        m.close()
    return out


def fem_small(flush, stream):
    """The 200x50 Q4 plane-stress operator (20 000 DOFs,
    BCSR bs 2, FP64). SpMV with x uniform in [-1, 1] (seed 0) on the GPU
    (warm: 3.5 MB stays in L2, as in the reference's own back-to-back timing;
    and L2-flushed) and on the host (the reference CPU loop, 1 thread and all
    threads), then the FP64 BiCGStab solve to 1e-10 on both."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from oracle import oracle as orc
    nx, ny = 200, 50
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    n = 2 * nx * ny
    x = bm.gen_uniform_vector(n, 0, X_STREAM)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    dx, dy = torch.from_numpy(x).cuda(), torch.empty(n, dtype=torch.float64, device="cuda")
    lanes = A.autotune(dx, dy)
    nbytes = bm.bcsr_spmv_bytes(np.float64, nx * ny, nx * ny, 2, int(c.size))
    warm_s = replay_seconds(lambda: A.spmv(dx, dy), 100, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cold = []
    for r in range(23):
        flush()
        e0.record(stream)
        A.spmv(dx, dy)
        e1.record(stream)
        e1.synchronize()
        if r >= 3:
            cold.append(e0.elapsed_time(e1) * 1e-3)
    cold_s = sum(cold) / len(cold)
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    y_ref = orc.csr_spmv(crp, cc, cv, x)
    err = float(np.sum((dy.cpu().numpy() - y_ref) ** 2) / np.sum(y_ref ** 2))
    threads = os.cpu_count() or 1
    cpu = {}
    for th in (1, threads):
        yb = np.zeros_like(x)
        orc.csr_spmv(crp, cc, cv, x, threads=th, out=yb)
        t0 = time.perf_counter()
        for _ in range(50):
            orc.csr_spmv(crp, cc, cv, x, threads=th, out=yb)
        sec = (time.perf_counter() - t0) / 50
        cpu[f"threads_{th}"] = {"us": round(sec * 1e6, 2), "gbs": round(nbytes / sec / 1e9, 2)}
    sv = bm.Solver(A, "fp64", tol=1e-10, max_iters=100000)
    d_b = torch.from_numpy(rhs).cuda()
    d_x = torch.empty_like(d_b)
    infos = [sv.solve(d_b, d_x) for _ in range(3)]
    sv.close()
    best = min(infos, key=lambda i: i["seconds"])
    xs = d_x.cpu().numpy()
    gpu_solve = {k: best[k] for k in ("iterations", "seconds", "true_rel_residual", "restarts", "replacements",
                                      "status")}
    gpu_solve["fp64_floor"] = fp64_floor(rp, c, v, 2, xs, rhs)
    gpu_solve["us_per_iteration"] = round(best["seconds"] / max(best["iterations"], 1) * 1e6, 2)
    A.close()
    return {"workload": "Q4 plane stress 200x50 nodes (E=1, nu=0.3, left edge clamped, f_y=-1 on the right edge), "
                        "20000 DOFs, BCSR bs 2, FP64",
            "nnzb": int(c.size), "spmv_bytes": int(nbytes), "lanes": lanes,
            "gpu_spmv": {"warm_us": round(warm_s * 1e6, 3), "warm_gbs": round(nbytes / warm_s / 1e9, 1),
                         "l2_flushed_us": round(cold_s * 1e6, 3), "l2_flushed_gbs": round(nbytes / cold_s / 1e9, 1),
                         "compare_results_error": err,
                         "note": "3.5 MB: launch- and latency-bound, not an HBM roofline case"},
            "cpu_spmv": cpu, "gpu_solve": gpu_solve,
            "cpu_solve": {"threads_1": cpu_solve((nx, ny), 1), f"threads_{threads}": cpu_solve((nx, ny), threads)}}


def iteration_roofline(grid, hbm_gbs, fp64_gflops, iters=300):
    """Live cost of one FP64 BiCGStab iteration of the whole-GPU engine on
    the Q4 operator (the auto launch mode's, with the graph of phase kernels
    and the persistent kernel beside it), against its two floors: HBM bytes (2 SpMV + 17 n vector
    elements of 8 bytes) over the measured copy bandwidth, and FP64 FMAs
    (8 per block for the two bs-2 products, 12 per row for the epilogue dots
    and vector updates) over the measured FP64 rate. Times `iters`
    iterations of one solve (the tolerance set out of reach)."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    nx, ny = grid
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    n, nnzb = 2 * nx * ny, int(c.size)
    d_b = torch.from_numpy(rhs).cuda()
    d_x = torch.empty_like(d_b)
    per_mode = {}
    for mode in ("graph", "persistent", "auto"):
        sv = bm.Solver(A, "fp64", tol=1e-30, max_iters=iters, launch_mode=mode)
        sv.solve(d_b, d_x)
        info = min((sv.solve(d_b, d_x) for _ in range(2)), key=lambda i: i["seconds"])
        sv.close()
        per_mode[mode] = info["seconds"] / max(info["iterations"], 1) * 1e6
    A.close()
    us = per_mode["auto"]
    nbytes = 2 * bm.bcsr_spmv_bytes(np.float64, nx * ny, nx * ny, 2, nnzb) + 17 * n * 8
    fmas = 8 * nnzb + 12 * n
    hbm_us = nbytes / (hbm_gbs * 1e9) * 1e6
    fp64_us = 2 * fmas / (fp64_gflops * 1e9) * 1e6
    floor = max(hbm_us, fp64_us)
    return {"grid": [nx, ny], "dofs": n, "iterations_timed": info["iterations"], "us_per_iteration": round(us, 2),
            "graph_us": round(per_mode["graph"], 2), "persistent_us": round(per_mode["persistent"], 2),
            "bytes_per_iteration": int(nbytes), "fp64_fmas_per_iteration": int(fmas),
            "hbm_floor_us": round(hbm_us, 2), "fp64_floor_us": round(fp64_us, 2),
            "floor_us": round(floor, 2), "of_floor": round(floor / us, 3)}


def precond_compare(grids, n_rhs=3, tol=1e-10, max_iters=200000):
    """FP64 BiCGStab on the Q4 operator with no preconditioner, point
    Jacobi (gpu/bicgstab.cu:201-238) and block Jacobi (the 2x2 diagonal
    blocks inverted), on the load vector and n_rhs - 1 seeded random loads
    (uniform in [-1, 1), 0 on the clamped column): iterations, seconds and
    true residual per right-hand side, and the medians. BiCGStab's
    iteration count on these ill-conditioned operators moves with any
    change of rounding, so one right-hand side says little."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    out = {}
    for nx, ny in grids:
        rp, c, v, load = bm.gen_q4_elasticity(nx, ny)
        A = bm.Matrix.from_bcsr(rp, c, v, 2)
        rng = np.random.default_rng(11)
        rhs = [load]
        for _ in range(n_rhs - 1):
            b = rng.uniform(-1, 1, 2 * nx * ny)
            b.reshape(ny, nx, 2)[:, 0, :] = 0.0
            rhs.append(b)
        res = {}
        for pre in ("none", "jacobi", "block_jacobi"):
            sv = bm.Solver(A, "fp64", tol=tol, max_iters=max_iters, preconditioner=pre)
            its, secs, rels = [], [], []
            for b in rhs:
                d_b = torch.from_numpy(b).cuda()
                d_x = torch.empty_like(d_b)
                info = sv.solve(d_b, d_x)
                its.append(info["iterations"])
                secs.append(round(info["seconds"], 4))
                rels.append(info["true_rel_residual"])
            sv.close()
            res[pre] = {"iterations": its, "seconds": secs, "true_rel": rels,
                        "median_iterations": float(np.median(its)), "median_seconds": float(np.median(secs))}
        out[f"{nx}x{ny}"] = res
        A.close()
    return out


def fem_large(cpu_iters=(12, 60)):
    """The Q4 operator on 2000x500 nodes (2 M DOFs, BCSR
    bs 2). Plain FP64 BiCGStab and FP32-inner / FP64-refined, both to 1e-10
    relative residual: iterations, time, true residual, the FP64 floor, and
    the mixed solution's error against the FP64 one. The CPU baseline runs
    the same recurrences for a bounded number of iterations (1 thread and all
    threads) and projects the GPU's iteration count at that rate."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from oracle import oracle as orc
    nx, ny = 2000, 500
    rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    d_b = torch.from_numpy(rhs).cuda()
    out, xs = {}, {}
    for prec in ("fp64", "mixed"):
        t0 = time.perf_counter()
        sv = bm.Solver(A, prec, tol=1e-10, max_iters=200000)
        setup = time.perf_counter() - t0
        d_x = torch.empty_like(d_b)
        info = sv.solve(d_b, d_x)
        sv.close()
        xs[prec] = d_x.cpu().numpy()
        out[prec] = {k: info[k] for k in ("iterations", "iterations_fp32", "seconds", "true_rel_residual", "restarts",
                                          "replacements", "used_fp64_fallback", "status")}
        out[prec]["setup_s"] = round(setup, 3)
        out[prec]["fp64_floor"] = fp64_floor(rp, c, v, 2, xs[prec], rhs)
        out[prec]["us_per_iteration"] = round(info["seconds"] / max(info["iterations"], 1) * 1e6, 2)
    out["mixed_error_vs_fp64"] = float(np.linalg.norm(xs["mixed"] - xs["fp64"]) / np.linalg.norm(xs["fp64"]))
    out["mixed_speedup"] = round(out["fp64"]["seconds"] / out["mixed"]["seconds"], 3)
    A.close()
    crp, cc, cv = orc.bcsr_to_csr(rp, c, v, 2)
    del rp, c, v
    threads = os.cpu_count() or 1
    cpu = {}
    for th, k in zip((1, threads), cpu_iters):
        t0 = time.perf_counter()
        if th == 1:
            _, st, it, rel = orc.bicgstab(crp, cc, cv, rhs, 1e-30, k)
        else:
            _, st, it, rel = orc.bicgstab_mt(crp, cc, cv, rhs, 1e-30, k, th)
        sec = time.perf_counter() - t0
        per_it = sec / max(it, 1)
        cpu[f"threads_{th}"] = {"iterations_timed": it, "s_per_iteration": round(per_it, 5),
                                "projected_solve_s": round(per_it * out["fp64"]["iterations"], 1)}
    out["cpu_solve"] = cpu
    out["cpu_solve"]["note"] = ("the reference recurrences (oracle.c) run for a bounded number of iterations; "
                                "projected_solve_s = s_per_iteration x the GPU FP64 solve's iterations")
    out["workload"] = "Q4 plane stress 2000x500 nodes, 2000000 DOFs, BCSR bs 2, nnzb 8985004"
    return out


def run_batch(args):
    from block_matrix_format_performance_gb300 import build as B
    B.build()
    grid = tuple(int(t) for t in args.batch_grid.lower().split("x")) if args.batch_grid else None
    shift = args.shift if args.matrix == "shifted" else None
    config = tuple(int(t) for t in args.batch_config.lower().split("x")) if args.batch_config else None
    res = measure_batch([args.precision], args.tol, args.max_iters, args.repeats, args.systems,
                        per_request=args.repeats > 0, grid=grid, shift=shift, config=config)
    print(json_line({"workload": "batch", "precision": args.precision,
                      "matrix": "q4" if shift is None else f"q4+{shift:g}I", **res}), flush=True)


def serve_stream(n_requests, rate, seed=1, large_fraction=0.05):
    """Seeded request stream: Poisson arrivals, grids as the uneven batch plus
    5 % 1000 x 250, right-hand sides uniform in [-1, 1) (0 on clamped DOFs)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    nxs = np.round(np.exp(rng.uniform(np.log(20), np.log(400), n_requests))).astype(int)
    big = rng.random(n_requests) < large_fraction
    grids = [(1000, 250) if bg else (int(nx), max(2, int(round(nx / 4)))) for nx, bg in zip(nxs, big)]
    return arrivals, grids


def serve_inputs(n_requests, rate, large_fraction, matrix="q4", shift=1e-3, seed=1):
    """The request stream (serve_stream), its distinct matrices as device
    handles and every request's right-hand side (uniform in [-1, 1), 0 on
    the clamped column)."""
    import block_matrix_format_performance_gb300 as bm
    arrivals, grids = serve_stream(n_requests, rate, seed=seed, large_fraction=large_fraction)
    mats = {}
    for g in sorted(set(grids)):
        rp, c, v, _ = shifted_q4(*g, shift) if matrix == "shifted" else bm.gen_q4_elasticity(*g)
        mats[g] = bm.Matrix.from_bcsr(rp, c, v, 2)
    rng = np.random.default_rng(7)
    rhs = []
    for nx, ny in grids:
        b = rng.uniform(-1, 1, 2 * nx * ny)
        b.reshape(ny, nx, 2)[:, 0, :] = 0.0  # clamped column carries no load
        rhs.append(b)
    return arrivals, grids, mats, rhs


def serve_once(precision, arrivals, grids, mats, rhs, tol, max_iters, **kw):
    """One pass of the stream through the continuous-batching server:
    requests submitted at their arrival times from a producer thread,
    latency = submit to completion (bmfp_solve_info.seconds)."""
    import threading

    import block_matrix_format_performance_gb300 as bm
    xs = [np.zeros_like(b) for b in rhs]
    srv = bm.Server(precision, tol=tol, max_iters=max_iters, **kw)
    small = min(mats)
    w = np.zeros(mats[small].rows)
    srv.wait(srv.submit(mats[small], np.ones_like(w), w))  # warm-up
    tickets = [None] * len(grids)
    t_start = time.perf_counter()

    def producer():
        for k, (t_arr, g) in enumerate(zip(arrivals, grids)):
            delay = t_arr - (time.perf_counter() - t_start)
            if delay > 0:
                time.sleep(delay)
            tickets[k] = srv.submit(mats[g], rhs[k], xs[k])

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    infos = [srv.wait(t) for t in tickets]
    makespan = time.perf_counter() - t_start
    stats = srv.stats()
    opts = {"wide_lanes": srv.options.wide_lanes, "wide_threshold_rows": srv.options.wide_threshold_rows}
    srv.close()
    lat = np.array([i["seconds"] for i in infos])
    bad = [{"grid": list(grids[k]), "status": i["status"], "true_rel": i["true_rel_residual"]}
           for k, i in enumerate(infos) if i["status"] != 0]
    return {"precision": precision, "requests": len(grids), "makespan_s": round(makespan, 3),
            "solves_per_s": round(len(grids) / makespan, 2),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4),
            "converged": sum(i["status"] == 0 for i in infos),
            "worst_true_rel": max(i["true_rel_residual"] for i in infos),
            "iterations": sum(i["iterations"] for i in infos),
            "iterations_fp32": sum(i["iterations_fp32"] for i in infos),
            "micro_batches": stats["micro_batches"], "wide_solves": stats["wide_solves"],
            "peak_device_bytes": stats["peak_bytes"], **opts, "not_converged": bad[:12]}, xs


def fifo_baseline(arrivals, grids, mats, rhs, tol, max_iters):
    """The plain FP64 per-request solver (the reference's path: one
    gpu_bicgstab solve per request, gpu/bicgstab.cu:387-526, here the
    whole-GPU engine) serving the stream first in, first out in real time:
    each request waits for its arrival and for the request before it, then
    its own right-hand side goes to the device, is solved, and x comes back.
    One solver per distinct matrix is built before the stream starts
    (setup_s). Returns the summary and every request's service time."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    t0 = time.perf_counter()
    solvers = {g: bm.Solver(m, "fp64", tol=tol, max_iters=max_iters) for g, m in mats.items()}
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    service, lat, infos = [], [], []
    t_start = time.perf_counter()
    for k, g in enumerate(grids):
        now = time.perf_counter() - t_start
        if arrivals[k] > now:
            time.sleep(arrivals[k] - now)
        s0 = time.perf_counter()
        d_b = torch.from_numpy(rhs[k]).cuda()
        d_x = torch.empty_like(d_b)
        infos.append(solvers[g].solve(d_b, d_x))
        d_x.cpu()
        s1 = time.perf_counter()
        service.append(s1 - s0)
        lat.append(s1 - t_start - arrivals[k])
    makespan = time.perf_counter() - t_start
    for sv in solvers.values():
        sv.close()
    return {"setup_s": round(setup, 3), "makespan_s": round(makespan, 3),
            "solves_per_s": round(len(grids) / makespan, 2),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4),
            "converged": sum(i["status"] == 0 for i in infos)}, service


def fifo_timeline(arrivals, service):
    """FIFO completion times of one server with the given service times:
    done_k = max(done_{k-1}, arrival_k) + service_k."""
    done, lat = 0.0, []
    for a, sv in zip(arrivals, service):
        done = max(done, a) + sv
        lat.append(done - a)
    return {"makespan_s": round(done, 3), "solves_per_s": round(len(arrivals) / done, 2),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4)}


def serve_suite(n_requests, rate, precisions, sustained_factor, tol=1e-10, max_iters=100000, large_fraction=0.05,
                sustained_requests=None):
    """The served request stream in the bench line: the stream at the stated rate
    through the server in each precision; the same requests at a rate the
    server sustains (sustained_factor x the first server's throughput at
    the stated rate, so that arrivals do not outrun it; the same exponential
    draws rescaled); and the plain FP64 per-request solver serving the
    stated-rate stream FIFO, every request solved in real time (the
    sustained stream's FIFO latencies follow from the same requests'
    measured service times)."""
    arrivals, grids, mats, rhs = serve_inputs(n_requests, rate, large_fraction)
    out = {"workload": f"Poisson arrivals, {n_requests} requests, grids as the uneven batch plus "
                       f"{large_fraction:.0%} 1000x250, random loads, tol {tol:g}, 120 GB HBM budget",
           "large_requests": int(sum(g == (1000, 250) for g in grids))}
    for prec in precisions:
        res, _ = serve_once(prec, arrivals, grids, mats, rhs, tol, max_iters)
        res["rate_req_s"] = rate
        out[f"served_{prec}_at_{rate:g}"] = res
    first = out[f"served_{precisions[0]}_at_{rate:g}"]
    sus_rate = round(sustained_factor * first["solves_per_s"], 1)
    ns = sustained_requests or n_requests
    sus_arr = arrivals[:ns] * (rate / sus_rate)
    res, _ = serve_once(precisions[0], sus_arr, grids[:ns], mats, rhs[:ns], tol, max_iters)
    res["rate_req_s"] = sus_rate
    out[f"served_{precisions[0]}_sustained"] = res
    base, service = fifo_baseline(arrivals, grids, mats, rhs, tol, max_iters)
    base["rate_req_s"] = rate
    out[f"fifo_plain_fp64_at_{rate:g}"] = base
    sus = fifo_timeline(sus_arr, service[:ns])
    sus["rate_req_s"] = sus_rate
    sus["note"] = "FIFO timeline of the same requests' measured service times"
    out["fifo_plain_fp64_sustained"] = sus
    for m in mats.values():
        m.close()
    return out


def run_serve(args):
    """Served solve stream through the continuous-batching server, and the
    same stream on the plain FP64 per-request solver (FIFO, every request
    solved)."""
    from block_matrix_format_performance_gb300 import build as B
    B.build()
    arrivals, grids, mats, rhs = serve_inputs(args.requests, args.rate, args.large_fraction, args.matrix, args.shift)
    kw = {}
    if args.wide_lanes is not None:
        kw["wide_lanes"] = args.wide_lanes
    if args.wide_threshold is not None:
        kw["wide_threshold_rows"] = args.wide_threshold
    if args.cluster_size is not None:
        kw["cluster_size"] = args.cluster_size
    if args.threads_per_cta is not None:
        kw["threads_per_cta"] = args.threads_per_cta
    if args.ctas_per_sm:
        kw["ctas_per_sm"] = args.ctas_per_sm
    res, _ = serve_once(args.precision, arrivals, grids, mats, rhs, args.tol, args.max_iters, **kw)
    base = None
    if not args.no_baseline:
        base, _ = fifo_baseline(arrivals, grids, mats, rhs, args.tol, args.max_iters)
    for m in mats.values():
        m.close()
    print(json_line({"workload": "serve", "matrix": "q4" if args.matrix == "q4" else f"q4+{args.shift:g}I",
                     "rate_req_s": args.rate, "tol": args.tol,
                     "large_requests": int(sum(g == (1000, 250) for g in grids)),
                     **res, "per_request_fp64": base}), flush=True)


def measure_variants(rp, c, v, bs, x, runs, stream):
    """Every SpMV format of the reference on one BCSR matrix (perform_measurements,
    main.cpp:131-148): "CPU CSR" is the single-thread CPU loop (main.cpp:21-63)
    through the oracle's restatement; each GPU format is checked against it
    with compare_results' rule (sum (a-b)^2 / sum b^2 <= 1e-9,
    measurement_class.h:58-87) and timed over `runs` launches replayed from a
    CUDA graph between CUDA events (replay_seconds; the reference records
    events around each launch, which here would time the host's launch
    latency).
    Returns ({format: mean seconds}, worst compare_results error)."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from oracle import oracle as orc
    n = x.size
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, bs)
    vt = bm.transpose_blocks(rp, v, bs)
    res = {}
    y_ref = orc.csr_spmv(crp, cc, cv, x)
    t0 = time.perf_counter()
    for _ in range(runs):
        orc.csr_spmv(crp, cc, cv, x)
    res["CPU CSR"] = (time.perf_counter() - t0) / runs
    d = {k: torch.from_numpy(a).cuda() for k, a in
         (("rp", rp), ("c", c), ("v", v), ("vt", vt), ("crp", crp), ("cc", cc), ("cv", cv), ("x", x))}
    dy = torch.empty(n, dtype=d["x"].dtype, device="cuda")
    colown = v.dtype == np.float64 and bs in (2, 4, 8, 16, 32)
    worst = 0.0
    for var in range(bm.VARIANT_COUNT):
        name = bm.variant_name(var)

        def launch():
            if bm.variant_is_csr(var):
                bm.csr_spmv(var, d["crp"], d["cc"], d["cv"], d["x"], dy)
            elif var == bm.BCSR_NATIVE and colown:
                # as the C++ drop-in's gpu_bcsr_spmv runs the native format:
                # the column owner on the caller's transposed blocks
                bm.bcsr_spmv_colmajor(d["rp"], d["c"], d["vt"], d["x"], dy, bs)
            else:
                vals = d["vt"] if bm.variant_layout(var) == 1 else d["v"]
                bm.bcsr_spmv(var, d["rp"], d["c"], vals, d["x"], dy, bs)
        try:
            launch()
        except bm.BmfpError as e:
            if e.status == bm.ERROR_NOT_SUPPORTED:
                continue  # e.g. the power-of-two variant at other bs, as gpu_matrix_multiplier.cu:1226
            raise
        torch.cuda.synchronize()
        y = dy.cpu().numpy()
        err = float(np.sum((y.astype(np.float64) - y_ref) ** 2) / np.sum(y_ref.astype(np.float64) ** 2))
        worst = max(worst, err)
        if err > 1e-9:
            raise SystemExit(f"{name} bs {bs}: compare_results error {err:.3e}")
        res[name] = replay_seconds(launch, runs, stream)
    return res, worst


def replay_seconds(launch, runs, stream):
    """Mean device time of one launch: `runs` launches captured in a CUDA graph
    and replayed between one pair of events, so the host's launch latency
    (10 us and more through Python, longer than a small product) does not
    sit between them. Launch sequences that cannot be captured are timed
    back to back instead."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    graph = None
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(runs):
                launch()
        g.replay()
        torch.cuda.synchronize()
        graph = g
    except Exception:
        torch.cuda.synchronize()
    e0.record(stream)
    if graph is not None:
        graph.replay()
    else:
        for _ in range(runs):
            launch()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3 / runs


def run_ndiag(args, sizes=(2, 4, 8, 16, 32), blocks_per_row=6, runs=10):
    """The reference's default run (main.cpp:383-398 -> measure_diag_matrices,
    main.cpp:318-344): gen_n_diag_bcsr matrices (FP32 by default, 50 000 block
    rows, 6 blocks per row) for bs 2..32, every format timed `runs` times and
    averaged (perform_measurements, main.cpp:131-148), kernels only between
    CUDA events (see measure_variants). The output map
    {bs: {format: mean seconds}} is the layout of the reference's
    results/result.json, which its plot/plot.py reads; "CPU CSR" is the
    single-thread CPU loop (main.cpp:21-63), timed through the oracle's
    restatement as the CPU baseline, and each GPU result is checked against it
    with compare_results' rule (sum (a-b)^2 / sum b^2 <= 1e-9,
    measurement_class.h:58-87)."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from block_matrix_format_performance_gb300 import build as B
    from oracle import oracle as orc
    B.build()
    orc.build()
    dt = np_dt(args.ndiag_dtype)
    n_rows = args.ndiag_rows
    results, checks = {}, {}
    stream = torch.cuda.current_stream()
    for bs in sizes:
        rp, c, v = bm.gen_n_diag_bcsr(n_rows, blocks_per_row, bs, dt)
        x = np.ones(n_rows * bs, dtype=dt)  # main.cpp:27 sets x := 1
        results[str(bs)], checks[str(bs)] = measure_variants(rp, c, v, bs, x, runs, stream)
    if args.results_json:
        with open(args.results_json, "w") as f:
            json.dump(results, f, indent=2, sort_keys=True)
    best = {bs: min((k for k in r if k != "CPU CSR"), key=r.get) for bs, r in results.items()}
    print(json_line({"workload": f"ndiag {args.ndiag_dtype}: gen_n_diag_bcsr {n_rows} block rows x "
                                  f"{blocks_per_row} blocks, bs {list(sizes)}, {runs} runs per format",
                      "results": results, "fastest": best, "worst_compare_results": checks}), flush=True)


def run_bridge(args, runs=10):
    """The reference's bridge run (measure_golden_bridge, main.cpp:349-381, off
    in its main): the Golden Gate truss of main.cpp:352-365 (128 km main span,
    260 m towers, 7.62 m segments, FP64, bs 2) through every SpMV format, and
    its solve as main.cpp:373-374 does it: Jacobi-preconditioned BiCGStab,
    epsilon 0.8 on the recursive residual, 1000 iterations."""
    import torch

    import block_matrix_format_performance_gb300 as bm
    from block_matrix_format_performance_gb300 import build as B
    from oracle import oracle as orc
    B.build()
    orc.build()
    t0 = time.perf_counter()
    rp, c, v, rhs = bm.gen_golden_gate_bridge(args.bridge_main_span, 345.0, 260.0, 7.62, 450.0, -2e6)
    gen_s = time.perf_counter() - t0
    n = rp.size - 1
    x = np.ones(2 * n)  # main.cpp:27 sets x := 1
    res, worst = measure_variants(rp, c, v, 2, x, runs, torch.cuda.current_stream())
    if args.results_json:
        with open(args.results_json, "w") as f:
            json.dump({"2": res}, f, indent=2, sort_keys=True)
    A = bm.Matrix.from_bcsr(rp, c, v, 2)
    s = bm.Solver(A, "fp64", tol=0.8, max_iters=1000, preconditioner="jacobi", check_true_residual=False)
    d_b = torch.from_numpy(rhs).cuda()
    d_x = torch.empty_like(d_b)
    s.solve(d_b, d_x)
    info = s.solve(d_b, d_x)
    s.close()
    A.close()
    best = min((k for k in res if k != "CPU CSR"), key=res.get)
    # the reference's stop rule leaves the true residual unevaluated (NaN): null in JSON
    info = {k: (None if isinstance(v, float) and v != v else v) for k, v in info.items()}
    print(json_line({"workload": "bridge", "main_span_m": args.bridge_main_span, "block_rows": n,
                      "nnzb": int(c.size), "generate_s": round(gen_s, 3), "spmv_seconds": res, "fastest": best,
                      "worst_compare_results": worst,
                      "solve": {"epsilon": 0.8, "max_iterations": 1000, "preconditioner": "jacobi", **info}}),
          flush=True)


def main():
    args = parse_args()
    if args.workload == "bridge":
        run_bridge(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "solve":
        run_solve(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "precond":
        from block_matrix_format_performance_gb300 import build as B
        B.build()
        grid = tuple(int(t) for t in args.grid.lower().split("x"))
        print(json_line({"workload": "precond", **precond_compare([grid], args.rhs, args.tol, args.max_iters)}),
              flush=True)
        return
    if args.workload == "ndiag":
        run_ndiag(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
