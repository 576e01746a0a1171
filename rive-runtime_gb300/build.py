"""Builds the product library librive_cuda.so (sm_103a) in-tree.

nvcc compiles each translation unit in parallel with one -gencode
(compute_103a -> sm_103a); the result lands in rive-runtime_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "librive_cuda.so")
SOURCES = ["context.cu", "kernels_tess.cu", "kernels_raster.cu", "flush_noalloc.cu"]
HEADERS = ["rive_cuda_internal.cuh", "rive_fp32_math.h"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code unfused (-ffp-contract=off): the feather tables it generates must
# round the same on x86 and Arm.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I" + os.path.join(REPO, "include"), "-I" + CSRC]
# The draw pass is compiled without contracting multiplies and adds into fused
# multiply-adds: its colour arithmetic (blend formulas, dither noise, the
# final blend) then rounds as the C restatement of the pass rounds it, so the
# few pixels where a last bit decides a unorm8 step, and chains of advanced
# blends amplify it, agree too. The hot loops use explicit fma intrinsics,
# which this leaves alone.
PER_SOURCE_FLAGS = {"kernels_raster.cu": ["--fmad=false"]}


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(REPO, "include", "rive_cuda.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs + [os.path.abspath(__file__)]):
            jobs.append([NVCC, *ARCH, *FLAGS, *PER_SOURCE_FLAGS.get(src, []), *extra_flags, "-c", s,
                         "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode:
                sys.stderr.write(res.stdout + res.stderr)
            if res.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if _stale(LIB, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
