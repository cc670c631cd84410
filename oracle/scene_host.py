"""The seeded benchmark scenes and camera matrices on the host alone.  BASELINE INFRASTRUCTURE ONLY.

The CPU arms of bench.py (the timed CPU baseline and --impl reference) need the same scenes and cameras as the GPU
arm without loading the CUDA library: this module binds oracle/_build/libscenehost.so, the product's generator
source (final184_gb300/csrc/scene.cpp) compiled on its own.  Structures are declared here independently.
"""
import ctypes as C

import numpy as np

from . import Bounds, Light
from . import build as _build

_lib = None


class _Scene(C.Structure):
    _fields_ = [("ntris", C.c_uint64), ("nobjects", C.c_uint32), ("pad", C.c_uint32),
                ("tri_xyz", C.POINTER(C.c_float)), ("albedo", C.POINTER(C.c_uint32)),
                ("roughness", C.POINTER(C.c_float)), ("object_first", C.POINTER(C.c_uint32)),
                ("object_count", C.POINTER(C.c_uint32)), ("bounds", Bounds), ("light", Light),
                ("eye", C.c_float * 3), ("target", C.c_float * 3)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build_scene_host())
        P = C.c_void_p
        _lib.f184gi_scene_generate.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(C.POINTER(_Scene))]
        _lib.f184gi_scene_free.argtypes = [C.POINTER(_Scene)]
        _lib.f184gi_scene_camera.argtypes = [C.POINTER(_Scene), C.c_uint64, C.c_uint32, P, P]
        _lib.f184gi_camera_perspective.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, P]
        _lib.f184gi_camera_look_at.argtypes = [P, P, P]
    return _lib


class HostScene:
    """The same fields as final184_gb300.SyntheticScene (numpy copies)."""

    def __init__(self, seed, target_tris, nobjects):
        ptr = C.POINTER(_Scene)()
        rc = lib().f184gi_scene_generate(seed, target_tris, nobjects, C.byref(ptr))
        if rc != 0:
            raise RuntimeError("scene generation failed (%d)" % rc)
        s = ptr.contents
        n = int(s.ntris)
        self.seed, self.ntris, self.nobjects = seed, n, int(s.nobjects)
        self.bounds, self.light = s.bounds, s.light
        self.eye = np.array(s.eye, dtype=np.float32)
        self.target = np.array(s.target, dtype=np.float32)
        self.tri_xyz = np.ctypeslib.as_array(s.tri_xyz, shape=(n * 9,)).copy()
        self.albedo = np.ctypeslib.as_array(s.albedo, shape=(n,)).copy()
        self.roughness = np.ctypeslib.as_array(s.roughness, shape=(n,)).copy()
        no = self.nobjects
        self.object_first = np.ctypeslib.as_array(s.object_first, shape=(no,)).copy()
        self.object_count = np.ctypeslib.as_array(s.object_count, shape=(no,)).copy()
        self._ptr = ptr

    def camera(self, i, seed=None):
        eye, tgt = (C.c_float * 3)(), (C.c_float * 3)()
        lib().f184gi_scene_camera(self._ptr, self.seed if seed is None else seed, i, eye, tgt)
        return np.array(eye, dtype=np.float32), np.array(tgt, dtype=np.float32)

    def __del__(self):
        try:
            if self._ptr:
                lib().f184gi_scene_free(self._ptr)
                self._ptr = None
        except Exception:
            pass


def perspective(fovy_deg, aspect, near, far):
    out = (C.c_float * 16)()
    lib().f184gi_camera_perspective(fovy_deg, aspect, near, far, out)
    return np.array(out, dtype=np.float32).reshape(4, 4)


def look_at(eye, target):
    out = (C.c_float * 16)()
    e = (C.c_float * 3)(*[float(x) for x in eye])
    t = (C.c_float * 3)(*[float(x) for x in target])
    lib().f184gi_camera_look_at(e, t, out)
    return np.array(out, dtype=np.float32).reshape(4, 4)
