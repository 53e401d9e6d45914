"""Host (CPU) builds of the device arithmetic headers for the CPU tests.

The CUDA kernels include csrc/ccd_math.h, ccd_ctcd64.h and ccd_cull32.h; the
same headers compile as plain C++ here so their arithmetic can be checked
against the oracle without a GPU.  These libraries are test instruments only.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "collisiondetection_gb300", "csrc")


def _build(name: str, src: str) -> str:
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, f"lib{name}.so")
    deps = [os.path.join(HERE, src)] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    if not os.path.exists(so) or any(os.path.getmtime(d) > os.path.getmtime(so) for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", so,
                        os.path.join(HERE, src)], check=True)
    return so


def math_lib():
    return ctypes.CDLL(_build("hc_math", "hostcheck_math.cpp"))


def core_lib():
    return ctypes.CDLL(_build("hc_core", "hostcheck_core.cpp"))
