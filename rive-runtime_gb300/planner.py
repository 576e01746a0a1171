"""ctypes binding of the host front end (include/rive_planner.h).

plan(scene_bytes) runs the planner on a rive_scene.h recording and returns the
frame's flush records as a capture.Capture, ready for rive_cuda.Context.render.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build
from . import capture

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.PLANNER_LIB):
            _build.build_planner()
        lib = ctypes.CDLL(_build.PLANNER_LIB)
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
