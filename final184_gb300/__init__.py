"""final184_gb300 -- GB300-native voxel cone-tracing GI path of Final184 (Python host bindings).

The compute path is libf184gi.so (hand-written sm_103a CUDA behind the C ABI in include/f184gi.h).  This module
is a thin ctypes layer that keeps the reference renderer's pass shape: a frame calls voxelize -> mip -> trace
(CMegaPipeline::Render, Foreground/Renderer/MegaPipeline.cpp:188-268).  Device buffers are passed as raw
device pointers (e.g. torch.Tensor.data_ptr()); streams as cudaStream_t handles (int) or None.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._abi import (FMT_F16, FMT_F32, FMT_RG16, GRID_KEEP_COUNTS, MarchParams, Bounds, ConeParams, F184Error, GridDesc, GridFrame, Light,
                   View, check, load)

__all__ = ["VoxelGI", "Grid", "SyntheticScene", "Light", "Bounds", "View", "ConeParams", "GridDesc", "GridFrame",
           "FMT_F32", "FMT_F16", "FMT_RG16", "GRID_KEEP_COUNTS", "MarchParams", "default_march_params", "F184Error", "perspective", "ortho", "look_at", "mat4_inverse",
           "make_light", "make_bounds", "default_cone_params", "frame_from_bounds", "make_view", "load"]


def _fa(values, n):
    return (C.c_float * n)(*[float(v) for v in np.asarray(values, dtype=np.float64).ravel()])


def perspective(fovy_deg, aspect, near, far):
    """CCamera::CalcPerspective (Foreground/SceneGraph/Camera.cpp:85-102), row-major 4x4."""
    out = (C.c_float * 16)()
    load().f184gi_camera_perspective(fovy_deg, aspect, near, far, out)
    return np.array(out, dtype=np.float32).reshape(4, 4)


def ortho(mag_x, mag_y, near, far):
    """CCamera::CalcOrtho (Camera.cpp:104-111), row-major 4x4."""
    out = (C.c_float * 16)()
    load().f184gi_camera_ortho(mag_x, mag_y, near, far, out)
    return np.array(out, dtype=np.float32).reshape(4, 4)


def look_at(eye, target):
    out = (C.c_float * 16)()
    load().f184gi_camera_look_at(_fa(eye, 3), _fa(target, 3), out)
    return np.array(out, dtype=np.float32).reshape(4, 4)


def mat4_inverse(m):
    out = (C.c_float * 16)()
    check(load().f184gi_mat4_inverse(_fa(m, 16), out))
    return np.array(out, dtype=np.float32).reshape(4, 4)


def make_light(luminance, direction):
    lt = Light()
    for i in range(3):
        lt.luminance[i] = float(luminance[i])
        lt.direction[i] = float(direction[i])
    return lt


def make_bounds(mn, mx):
    b = Bounds()
    b.min.x, b.min.y, b.min.z = (float(v) for v in mn)
    b.max.x, b.max.y, b.max.z = (float(v) for v in mx)
    return b


def frame_from_bounds(bounds, dim, light_dir):
    """Grid placement + light frame computed on the host (bit-identical to the device's)."""
    f = GridFrame()
    check(load().f184gi_frame_from_bounds(C.byref(bounds), dim, _fa(light_dir, 3), C.byref(f)))
    return f


def default_march_params():
    p = MarchParams()
    load().f184gi_march_params_default(C.byref(p))
    return p


def default_cone_params():
    p = ConeParams()
    load().f184gi_cone_params_default(C.byref(p))
    return p


class SyntheticScene:
    """Seeded scene (room + boxes/UV-spheres) owned by the library; arrays are numpy copies."""

    def __init__(self, seed, target_tris, nobjects, _ptr=None):
        lib = load()
        ptr = _ptr
        if ptr is None:
            ptr = C.POINTER(_abi.Scene)()
            check(lib.f184gi_scene_generate(seed, target_tris, nobjects, C.byref(ptr)))
        self._ptr = ptr
        s = ptr.contents
        self.seed = seed
        self.ntris = int(s.ntris)
        self.nobjects = int(s.nobjects)
        self.bounds = s.bounds
        self.light = s.light
        self.eye = np.array(s.eye, dtype=np.float32)
        self.target = np.array(s.target, dtype=np.float32)
        self._refresh()

    def _refresh(self):
        s = self._ptr.contents
        n = self.ntris
        self.tri_xyz = np.ctypeslib.as_array(s.tri_xyz, shape=(n * 9,)).copy()
        self.albedo = np.ctypeslib.as_array(s.albedo, shape=(n,)).copy()
        self.roughness = np.ctypeslib.as_array(s.roughness, shape=(n,)).copy()
        self.object_first = np.ctypeslib.as_array(s.object_first, shape=(self.nobjects,)).copy()
        self.object_count = np.ctypeslib.as_array(s.object_count, shape=(self.nobjects,)).copy()

    @classmethod
    def from_gltf(cls, path):
        """A glTF 2.0 file (.gltf / .glb) flattened to world-space triangles (f184gi_gltf_load)."""
        ptr = C.POINTER(_abi.Scene)()
        check(load().f184gi_gltf_load(str(path).encode(), C.byref(ptr)))
        return cls(0, 0, 0, _ptr=ptr)

    def camera(self, i, seed=None):
        eye = (C.c_float * 3)()
        tgt = (C.c_float * 3)()
        check(load().f184gi_scene_camera(self._ptr, self.seed if seed is None else seed, i, eye, tgt))
        return np.array(eye, dtype=np.float32), np.array(tgt, dtype=np.float32)

    def move_objects(self, seed, fraction, max_offset):
        moved = (C.c_uint32 * self.nobjects)()
        n = C.c_uint32()
        check(load().f184gi_scene_move_objects(self._ptr, seed, fraction, max_offset, moved, C.byref(n)))
        self._refresh()
        return np.array(moved[: n.value], dtype=np.uint32)

    def __del__(self):
        try:
            if self._ptr:
                load().f184gi_scene_free(self._ptr)
                self._ptr = None
        except Exception:
            pass


class Grid:
    def __init__(self, gi, handle, desc):
        self.gi = gi
        self.handle = handle
        self.desc = desc

    @property
    def dim(self):
        return self.desc.dim

    def level_dim(self, level):
        return self.desc.dim >> level


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return C.c_void_p(s.cuda_stream)
    return C.c_void_p(int(s))


class VoxelGI:
    """One f184gi context: resident grids plus the voxelize / mip / trace passes."""

    def __init__(self, device=0, hbm_budget=0):
        self.lib = load()
        cfg = _abi.Config(device, 0, hbm_budget)
        ctx = C.c_void_p()
        check(self.lib.f184gi_create(C.byref(cfg), C.byref(ctx)))
        self.ctx = ctx

    def close(self):
        if self.ctx:
            check(self.lib.f184gi_destroy(self.ctx))
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def memory_used(self):
        v = C.c_uint64()
        check(self.lib.f184gi_memory_used(self.ctx, C.byref(v)))
        return v.value

    def create_grid(self, dim, levels, fmt=FMT_F32, anisotropic=0, shadow_res=1024, flags=0):
        d = GridDesc(dim, levels, fmt, anisotropic, shadow_res, flags)
        h = C.c_uint32()
        check(self.lib.f184gi_grid_create(self.ctx, C.byref(d), C.byref(h)))
        return Grid(self, h.value, d)

    def destroy_grid(self, grid):
        check(self.lib.f184gi_grid_destroy(self.ctx, grid.handle))

    def voxelize(self, grid, tri_ptr, albedo_ptr, ntris, light, bounds=None, dirty_ptr=None, ndirty=0, stream=None):
        check(self.lib.f184gi_voxelize(self.ctx, grid.handle, tri_ptr, albedo_ptr, ntris,
                                       C.byref(bounds) if bounds is not None else None, C.byref(light),
                                       dirty_ptr, ndirty, _stream(stream)))

    def mip(self, grid, levels=0, stream=None):
        check(self.lib.f184gi_mip(self.ctx, grid.handle, levels, grid.desc.anisotropic, _stream(stream)))

    def trace(self, grid, views, params=None, stream=None):
        arr = (View * len(views))(*views)
        check(self.lib.f184gi_trace(self.ctx, grid.handle, arr, len(views),
                                    C.byref(params) if params is not None else None, _stream(stream)))

    def trace_count(self, grid, views, params=None, stream=None):
        """trace() through the instrumented kernel; returns (cone steps, level samples) over all pixels."""
        arr = (View * len(views))(*views)
        counts = (C.c_uint64 * 2)()
        check(self.lib.f184gi_trace_count(self.ctx, grid.handle, arr, len(views),
                                          C.byref(params) if params is not None else None, counts, _stream(stream)))
        return int(counts[0]), int(counts[1])

    def march(self, grid, views, params=None, stream=None):
        """The reference-faithful indirect pass over an RG16 grid (out: width*height RGBA FP32 per view)."""
        arr = (View * len(views))(*views)
        check(self.lib.f184gi_march(self.ctx, grid.handle, arr, len(views),
                                    C.byref(params) if params is not None else None, _stream(stream)))

    def blur(self, in_ptr, depth_ptr, width, height, out_ptr, stream=None):
        """The reference's depth-aware blur of an RGBA FP32 image (device pointers)."""
        check(self.lib.f184gi_blur(self.ctx, in_ptr, depth_ptr, width, height, out_ptr, _stream(stream)))

    def gbuffer(self, tri_ptr, rough_ptr, ntris, view, tri_id_ptr=None, stream=None):
        check(self.lib.f184gi_gbuffer(self.ctx, tri_ptr, rough_ptr, ntris, C.byref(view), tri_id_ptr,
                                      _stream(stream)))

    def sync(self, stream=None):
        check(self.lib.f184gi_sync(self.ctx, _stream(stream)))

    def selftest_bounded_wait(self, polls, complete, stream=None, as_copy_wait=False):
        """One bounded device wait that expires unless `complete`; the expiry surfaces at the next sync().
        as_copy_wait: the expiry is recorded as an expired bulk-copy wait, after which the context refuses calls."""
        check(self.lib.f184gi_selftest_bounded_wait(self.ctx, polls, 2 if as_copy_wait else (1 if complete else 0),
                                                    _stream(stream)))

    def frame(self, grid):
        f = GridFrame()
        check(self.lib.f184gi_grid_get_frame(self.ctx, grid.handle, C.byref(f)))
        return f

    def level_ptr(self, grid, level):
        """(device pointer, bytes) of one level of the chain (all six direction volumes of an anisotropic level).
        The caller may write through it: the next mip() then builds the whole chain from level 0."""
        ptr, nbytes = C.c_void_p(), C.c_uint64()
        check(self.lib.f184gi_grid_level_ptr(self.ctx, grid.handle, level, C.byref(ptr), C.byref(nbytes)))
        return int(ptr.value or 0), int(nbytes.value)

    def read_level(self, grid, level, direction=0):
        d = grid.level_dim(level)
        if grid.desc.format == FMT_RG16:  # packed uint32 per voxel (565 albedo | 565 normal << 16)
            out = np.empty((d, d, d), dtype=np.uint32)
            check(self.lib.f184gi_grid_read_level(self.ctx, grid.handle, level, direction, out.ctypes.data))
            return out
        out = np.empty((d, d, d, 4), dtype=np.float32)
        check(self.lib.f184gi_grid_read_level(self.ctx, grid.handle, level, direction, out.ctypes.data))
        return out

    def read_shadow(self, grid):
        r = grid.desc.shadow_res
        out = np.empty((r, r), dtype=np.float32)
        check(self.lib.f184gi_grid_read_shadow(self.ctx, grid.handle, out.ctypes.data))
        return out

    def read_counts(self, grid):
        d = grid.dim
        out = np.empty((d, d, d), dtype=np.uint32)
        check(self.lib.f184gi_grid_read_counts(self.ctx, grid.handle, out.ctypes.data))
        return out


def make_view(view_m, proj_m, width, height, depth_ptr, normal_ptr, rough_ptr, out_ptr, out_format=FMT_F32):
    v = View()
    for i, x in enumerate(np.asarray(view_m, dtype=np.float32).ravel()):
        v.view[i] = float(x)
    for i, x in enumerate(np.asarray(proj_m, dtype=np.float32).ravel()):
        v.proj[i] = float(x)
    v.width, v.height = width, height
    v.depth, v.normal, v.roughness, v.out = depth_ptr, normal_ptr, rough_ptr, out_ptr
    v.out_format = out_format
    return v


class Server:
    """Continuous-batching request server over device-resident scenes (f184gi_server_*)."""

    def __init__(self, device=0, slots=2, max_batch_views=64, blocks_per_sm=0, hbm_budget=0, cone=None,
                 trace_variant=None):
        """trace_variant None: tune the cone-trace kernel variant on the first batch; k: use variant k."""
        self.lib = load()
        cfg = _abi.ServerConfig(device, slots, max_batch_views, blocks_per_sm, hbm_budget,
                                cone if cone is not None else _abi.ConeParams(),
                                0 if trace_variant is None else trace_variant + 1, 0)
        h = C.c_void_p()
        check(self.lib.f184gi_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    def add_scene(self, scene_id, desc, tri_xyz, albedo, bounds, light):
        tri = np.ascontiguousarray(tri_xyz, dtype=np.float32)
        alb = np.ascontiguousarray(albedo, dtype=np.uint32)
        check(self.lib.f184gi_server_add_scene(self.h, scene_id, C.byref(desc), tri.ctypes.data, alb.ctypes.data,
                                               tri.size // 9, C.byref(bounds), C.byref(light)))

    def submit(self, scene_id, views, moves=(), host_buffers=False, flags=0):
        """flags: extra F184GI_REQ_* bits (e.g. the fault-injection test hooks _abi.REQ_INJECT_*)."""
        mv = (_abi.Move * max(1, len(moves)))(*[_abi.Move(int(f), int(c), (C.c_float * 3)(*o)) for f, c, o in moves])
        vw = (View * len(views))(*views)
        req = _abi.Request(scene_id, (_abi.REQ_HOST_BUFFERS if host_buffers else 0) | flags, mv, len(moves),
                           len(views), vw)
        t = C.c_uint64()
        check(self.lib.f184gi_server_submit(self.h, C.byref(req), C.byref(t)))
        return t.value

    def submit_many(self, requests, host_buffers=False):
        """Queue [(scene_id, views, moves[, flags]), ...] at once (one batch can take them all); returns the
        tickets."""
        keep, reqs = [], []
        for req in requests:
            scene_id, views, moves = req[:3]
            flags = req[3] if len(req) > 3 else 0
            mv = (_abi.Move * max(1, len(moves)))(*[_abi.Move(int(f), int(c), (C.c_float * 3)(*o))
                                                     for f, c, o in moves])
            vw = (View * len(views))(*views)
            keep += [mv, vw]
            reqs.append(_abi.Request(scene_id, (_abi.REQ_HOST_BUFFERS if host_buffers else 0) | flags, mv,
                                     len(moves), len(views), vw))
        arr = (_abi.Request * len(reqs))(*reqs)
        t = (C.c_uint64 * len(reqs))()
        check(self.lib.f184gi_server_submit_batch(self.h, arr, len(reqs), t))
        return list(t)

    def wait(self, ticket, timeout_ms=0):
        r = _abi.RequestResult()
        rc = self.lib.f184gi_server_wait(self.h, ticket, timeout_ms, C.byref(r))
        if rc != _abi.OK:
            raise F184Error(rc, self.lib.f184gi_last_error().decode())
        return r

    def cancel(self, ticket):
        check(self.lib.f184gi_server_cancel(self.h, ticket))

    def set_log(self, path):
        """Append one JSON line per finished request to `path` (None: stop)."""
        check(self.lib.f184gi_server_set_log(self.h, None if path is None else str(path).encode()))

    def stats(self):
        st = _abi.ServerStats()
        check(self.lib.f184gi_server_get_stats(self.h, C.byref(st)))
        return st

    def close(self):
        if self.h:
            check(self.lib.f184gi_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
