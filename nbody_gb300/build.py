"""Builds libnbody_gb300.so in-tree: one nvcc process per translation unit,
run in parallel, for sm_103a only, then linked with nvcc.

Usage: python -m nbody_gb300.build [--force] [--verbose]
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
UNITS = ["api.cu", "sort.cu", "tree.cu", "direct.cu", "direct_static.cu", "fmm_fp32.cu", "fmm_mixed.cu", "fmm_fp64.cu", "adjoint.cu", "lists.cu", "trajectory.cu"]
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


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
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
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
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
    if force or jobs or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
