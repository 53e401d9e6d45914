"""Builds the native library libccd_gb300.so in-tree (collisiondetection_gb300/_build/).

Every CUDA translation unit is compiled for sm_103a only, with
--fmad=false (the FP64 path reproduces the reference's one rounding per
operation; see csrc/ccd_common.h).  Units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libccd_gb300.so")

CU_SOURCES = ["narrow_vf.cu", "narrow_ee.cu", "narrow_vevv.cu", "narrow.cu", "stages.cu", "radix_sort.cu",
              "broadphase.cu", "mesh.cu", "capi.cu", "capi_mesh.cu",
              "capi_noalloc.cu", "capi_tune.cu", "server.cu", "distance.cu", "penalty.cu", "separating.cu", "velocity.cu"]
HEADERS = ["ccd_common.h", "ccd_math.h", "ccd_math_tables.h", "ccd_jt.h", "ccd_jt_warp.h", "ccd_jt_shifts.h", "ccd_ctcd64.h", "ccd_cull32.h", "narrow.cuh", "narrow_kernels.cuh", "stages.cuh",
           "radix_sort.cuh", "broadphase.cuh", "mesh.cuh", "context.cuh", "ccd_distance.h", "distance.cuh", "separating.cuh", "penalty.cuh", "velocity.cuh", "ccd_heap.h"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I" + os.path.join(ROOT, "include"),
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libccd_gb300.so")
    return path


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "ccd_gb300.h"),
                                                           os.path.abspath(__file__)]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, *objs])
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
