"""Builds libnbody_gb300.so in-tree: one nvcc process per translation unit,
run in parallel, for sm_103a only, then linked with nvcc.

With debug=True (--debug) it builds libnbody_gb300_debug.so instead: the same
sources with -DNBODY_DEBUG_BOUNDS, whose kernels check every index they read
from device data and report a failed check as an error (objects in
_build_debug/).

Usage: python -m nbody_gb300.build [--force] [--verbose] [--debug]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnbody_gb300.so")
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(HERE, "libnbody_gb300_debug.so")
UNITS = ["api.cu", "sort.cu", "tree.cu", "direct.cu", "direct_static.cu", "fmm_fp32.cu", "fmm_mixed.cu", "fmm_fp64.cu", "adjoint.cu", "lists.cu", "trajectory.cu", "blocksteps.cu"]
HEADERS = ["nbody_internal.cuh", "fmm_impl.cuh", "adjoint_impl.cuh", "fmm_ops.inc", "../../include/nbody_gb300.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None, debug: bool = False) -> str:
    bdir, lib = (BUILD_DEBUG, LIB_DEBUG) if debug else (BUILD, LIB)
    extra = list(extra or []) + (["-DNBODY_DEBUG_BOUNDS"] if debug else [])
    os.makedirs(bdir, exist_ok=True)
    gen = os.path.join(CSRC, "gen_ops.py")
    inc = os.path.join(CSRC, "fmm_ops.inc")
    if force or _stale(inc, [gen]):
        with open(inc, "w") as f:
            subprocess.run([sys.executable, gen], check=True, stdout=f)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    cc = nvcc()
    jobs = []
    objs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(bdir, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs + [__file__]):
            cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", src, "-o", obj]
            jobs.append((u, cmd))

    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for name, r in ex.map(run, jobs):
                if verbose or r.returncode != 0:
                    sys.stderr.write(f"== {name}\n{r.stdout}{r.stderr}")
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {name}")
    if force or jobs or _stale(lib, objs):
        cmd = [cc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv, debug="--debug" in sys.argv))
