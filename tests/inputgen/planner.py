"""TEST AND BENCH INFRASTRUCTURE: ctypes binding of the front-end stand-in
(rive_planner.h in this directory), which produces flush records where the
reference's own front end cannot be built.

plan(scene_bytes) runs it on a rive_scene.h recording and returns the frame's
flush records as a capture.Capture, ready for rive_cuda.Context.render.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

from rive_runtime_gb300 import capture

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
PLANNER_LIB = os.path.join(OUT, "librive_planner.so")
SOURCES = [os.path.join(HERE, "planner.cpp")]
CXX = os.environ.get("CXX", "g++")


def build(verbose=False):
    """Builds librive_planner.so: plain C++17, no CUDA; -ffp-contract=off keeps
    its float arithmetic identical across x86-64 and aarch64."""
    os.makedirs(OUT, exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "rive_planner.h")] + [
        os.path.join(REPO, "include", h) for h in ("rive_scene.h", "rive_cuda.h")]
    if os.path.exists(PLANNER_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(PLANNER_LIB)
                                           for d in deps):
        return PLANNER_LIB
    cmd = [CXX, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
           "-I" + HERE, "-I" + os.path.join(REPO, "include"), *SOURCES, "-o", PLANNER_LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or res.returncode:
        sys.stderr.write(res.stdout + res.stderr)
    if res.returncode:
        raise RuntimeError("planner build failed")
    return PLANNER_LIB

_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(PLANNER_LIB)
        lib.rive_plan_scene.restype = ctypes.c_int
        lib.rive_plan_scene.argtypes = [ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_void_p),
                                        ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.c_char_p, ctypes.c_size_t]
        lib.rive_plan_free.restype = None
        lib.rive_plan_free.argtypes = [ctypes.c_void_p]
        _lib = lib
    return _lib


def plan_bytes(scene_bytes: bytes) -> bytes:
    lib = load()
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    err = ctypes.create_string_buffer(512)
    rc = lib.rive_plan_scene(scene_bytes, len(scene_bytes), ctypes.byref(out),
                             ctypes.byref(n), err, 512)
    if rc != 0:
        raise RuntimeError(f"planner failed ({rc}): {err.value.decode()}")
    try:
        return ctypes.string_at(out, n.value)
    finally:
        lib.rive_plan_free(out)


def plan(scene_bytes: bytes) -> capture.Capture:
    return capture.parse(plan_bytes(scene_bytes))
