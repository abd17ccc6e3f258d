"""Builds libivr_gpu.so in-tree: the CUDA kernels for sm_103a and the C ABI.

Kernels are compiled with -fmad=false (every multiply and add rounded on
its own unless written as fmaf) and IEEE division/square root; host code
with -ffp-contract=off.  Both are what makes the REF preset bit-compatible
with the reference's C.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libivr_gpu.so")
# the reference's own names over LIB (include/ivr_compat.h)
COMPAT_SRC = os.path.join(HERE, "compat", "ivr_compat.c")
COMPAT_LIB = os.path.join(HERE, "libivr_compat.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CUDA_INC = os.path.join(os.path.dirname(os.path.dirname(NVCC)), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
            "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _run(cmd, log):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if log is not None:
        log.append((cmd, p.stdout + p.stderr))
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)


def build(verbose: bool = False) -> str:
    """Compiles every source and links the library; IVR_NVCC_EXTRA adds
    nvcc flags (for tuning builds)."""
    os.makedirs(BUILD, exist_ok=True)
    extra = os.environ.get("IVR_NVCC_EXTRA", "").split()
    cu, cpp = sources()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs, objs = [], []
    for f in cu:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([NVCC, *ARCH, *CU_FLAGS, *extra, *inc, "-c", os.path.join(CSRC, f), "-o", o])
    for f in cpp:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append(["g++", *CXX_FLAGS, *inc, "-I" + CUDA_INC, "-c", os.path.join(CSRC, f), "-o", o])
    log = []
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, log), jobs))
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"], log)
    os.replace(tmp, LIB)
    tmp = COMPAT_LIB + ".tmp"
    _run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-Wall", "-Wextra", "-Wno-unused-parameter",
          "-I" + os.path.join(ROOT, "include"), COMPAT_SRC, "-o", tmp, "-L" + HERE, "-l:libivr_gpu.so",
          "-Wl,-rpath,$ORIGIN"], log)
    os.replace(tmp, COMPAT_LIB)
    if verbose:
        for cmd, out in log:
            if out.strip():
                print(" ".join(os.path.basename(c) for c in cmd[:1]), out, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
