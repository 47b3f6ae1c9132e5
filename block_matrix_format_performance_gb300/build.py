"""Build libbmfp.so in-tree with nvcc for sm_103a (and g++ for host-only files).

    python -m block_matrix_format_performance_gb300.build [--force] [-v]

Every translation unit is compiled in parallel into ``_build/`` at the
repository root, then linked into ``block_matrix_format_performance_gb300/libbmfp.so``
against the CUDA runtime and cuSPARSE. A rebuild is skipped when the library
is newer than every source and header.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import fcntl
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libbmfp.so")

SOURCES = [
    "spmv_native.cu",
    "spmv_variants.cu",
    "spmv_host.cpp",
    "peaks.cu",
    "vector_ops.cu",
    "bicgstab.cu",
    "batch.cu",
    "noalloc.cu",
    "api.cpp",
    "solver_api.cpp",
    "serve.cpp",
    "cusparse.cpp",
    "host.cpp",
    "bridge.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env and os.path.isdir(env):
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _nvcc() -> str:
    return os.path.join(cuda_home(), "bin", "nvcc")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _compile_cmd(src: str, obj: str):
    path = os.path.join(CSRC, src)
    common_inc = ["-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        return [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", *common_inc,
                "-c", path, "-o", obj]
    cxx = os.environ.get("CXX", "g++")
    return [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
            "-pthread", "-Wall", "-Wno-unused-function", *common_inc,
            "-I", os.path.join(cuda_home(), "include"), "-c", path, "-o", obj]


def _newest_input() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for dp, _, files in os.walk(d):
            for f in files:
                t = max(t, os.path.getmtime(os.path.join(dp, f)))
    return max(t, os.path.getmtime(__file__))


def up_to_date() -> bool:
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link libbmfp.so; returns its path. Processes that build at
    the same time (one per rank under torchrun, parallel test workers) take
    turns on a lock file; the later ones find the library up to date."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with open(os.path.join(BUILD, ".lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and up_to_date():
            return LIB
        return _build_locked(verbose, jobs)


def _build_locked(verbose: bool, jobs: int | None) -> str:
    srcs = _sources()
    objs = [os.path.join(BUILD, s.replace(".", "_") + ".o") for s in srcs]
    cmds = [_compile_cmd(s, o) for s, o in zip(srcs, objs)]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        if verbose and (p.stdout or p.stderr):
            print(p.stdout + p.stderr, flush=True)

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + ".tmp"
    link = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lcusparse", "-lpthread"]
    run(link)
    os.replace(tmp, LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose))


if __name__ == "__main__":
    sys.exit(main())
