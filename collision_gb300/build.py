"""Build the CUDA library in-tree: collision_gb300/_build/libcollision_gb300.so.

Every translation unit is compiled for sm_103a only, in parallel, with
--fmad=false (no multiply-add contraction: the plain FP64 path rounds each
product and sum separately, as the reference's x86 build does) and the host
parts with -ffp-contract=off for the same reason on Arm hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcollision_gb300.so")
SOURCES = ["cc_prims.cu", "cc_bvh.cu", "cc_narrow.cu", "cc_post.cu", "cc_zones.cu", "cc_loop.cu", "cc_runtime.cu", "cc_noalloc.cu",
           "cc_tree_order.cpp", "cc_tree_gpu.cu", "cc_strain_plan.cpp", "cc_vtk.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "collision_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if force or _stale(obj, path):
            flags = list(NVCC_FLAGS)
            if ptxas_info and src.endswith(".cu"):
                flags += ["-Xptxas", "-v"]
            jobs.append([nv, *flags, "-c", path, "-o", obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out:
                    print(out)
    objs = [os.path.join(BUILD, s + ".o") for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nv, *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv))
