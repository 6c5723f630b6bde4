"""Build libgmhd.so (the CUDA kernels + C ABI) for sm_103a with nvcc, in-tree.

    python -m godunov_mhd_ct_gb300.csrc.build        (or build() from Python)

The FP64 unit is compiled with --fmad=false so its arithmetic matches the reference formulas'
FP64 rounding; the mixed unit keeps FMA contraction. Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libgmhd.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
UNITS = {
    "step_fp64.cu": ["--fmad=false"],
    "step_fp64_visc.cu": ["--fmad=false"],
    "step_mixed.cu": ["--use_fast_math"],
    "step_mixed_visc.cu": ["--use_fast_math"],
    "step_column.cu": ["--use_fast_math"],
    "gmhd_abi.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "amr.cu": ["--fmad=false"],
    "forest.cpp": ["-Xcompiler", "-pthread"],
}
HEADERS = ["mhd_math.cuh", "fused_step.cuh", "column_step.cuh", "launch.cuh",
           os.path.join("..", "..", "include", "gmhd.h")]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgmhd.so")
    return exe


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(HERE, h) for h in HEADERS]
    jobs = []
    for unit, flags in UNITS.items():
        src = os.path.join(HERE, unit)
        obj = os.path.join(OBJDIR, unit.rsplit(".", 1)[0] + ".o")
        if force or _stale(obj, [src, __file__] + headers):
            cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    objs = [os.path.join(OBJDIR, u.rsplit(".", 1)[0] + ".o") for u in UNITS]
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout + r.stderr)
            raise RuntimeError("nvcc link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
