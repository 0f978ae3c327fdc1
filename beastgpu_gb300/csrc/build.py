"""Build libbeastgb.so (the C-ABI library) for sm_103a with nvcc, in-tree.

Each .cu file is compiled in parallel, then linked into beastgpu_gb300/libbeastgb.so.
Usage: python -m beastgpu_gb300.csrc.build [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
OUT = os.path.join(PKG, "libbeastgb.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["bgb_api.cu", "bgb_plan.cu", "bgb_singular.cu", "bgb_far.cu", "bgb_peaks.cu", "bgb_noalloc.cu", "bgb_batch.cu", "bgb_singular_df.cu", "bgb_curve.cu"] + [
    f"bgb_far_{p}_op{o}.cu" for p in ("mixed", "fp64") for o in (0, 1, 2, 3, 4, 5)]
HEADERS = ["bgb_common.cuh", "bgb_kernels.cuh", "bgb_far_impl.cuh", "bgb_host.h", "bgb_df.cuh", "bgb_ss.cuh", "trirules.h", "besselfit.h", os.path.join("..", "..", "include", "beastgb.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(HERE, h) for h in HEADERS]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(HERE, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", s, "-o", o]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
            for cmd, fut in zip(jobs, futs):
                r = fut.result()
                if verbose or r.returncode:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or _stale(OUT, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", OUT + ".tmp", *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
