"""ctypes mirror of include/f184gi.h (structures and prototypes).

Loading fails loudly when the shared library has not been built: there is no Python fallback for any pass.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libf184gi.so")

FMT_F32 = 0
FMT_F16 = 1
FMT_RG16 = 2
GRID_KEEP_COUNTS = 1
GRID_RESIDENT_WEIGHTS = 2

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_OOM = -3
ERR_BUDGET = -4
ERR_OVERFLOW = -5
ERR_TIMEOUT = -6
ERR_NOTFOUND = -7
ERR_CANCELLED = -8
ERR_WORKER = -9
REQ_HOST_BUFFERS = 1
REQ_INJECT_FAIL = 0x100
REQ_INJECT_WORKER_EXIT = 0x200


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Bounds(C.Structure):
    _fields_ = [("min", Vec3), ("pad0", C.c_float), ("max", Vec3), ("pad1", C.c_float)]


class Light(C.Structure):
    _fields_ = [("luminance", C.c_float * 3), ("direction", C.c_float * 3)]


class GridDesc(C.Structure):
    _fields_ = [("dim", C.c_uint32), ("levels", C.c_uint32), ("format", C.c_uint32),
                ("anisotropic", C.c_uint32), ("shadow_res", C.c_uint32), ("flags", C.c_uint32)]


class GridFrame(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("voxel_size", C.c_double), ("inv_voxel_fixed", C.c_double),
                ("light_clip", C.c_double * 16), ("shadow_bias", C.c_double), ("light_dir", C.c_double * 3),
                ("light_vox", C.c_float * 12), ("shadow_bias_f", C.c_float), ("pad_f", C.c_float * 3)]


class View(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("width", C.c_uint32), ("height", C.c_uint32),
                ("depth", C.c_void_p), ("normal", C.c_void_p), ("roughness", C.c_void_p), ("out", C.c_void_p),
                ("out_format", C.c_uint32), ("pad", C.c_uint32)]


class ConeParams(C.Structure):
    _fields_ = [("diffuse_cones", C.c_uint32), ("diffuse_tan_half", C.c_float), ("diffuse_tilt_deg", C.c_float),
                ("step_factor", C.c_float), ("max_distance", C.c_float), ("alpha_stop", C.c_float),
                ("start_offset", C.c_float), ("min_spec_tan_half", C.c_float), ("specular", C.c_uint32),
                ("pad", C.c_uint32)]


class Move(C.Structure):
    _fields_ = [("first", C.c_uint32), ("count", C.c_uint32), ("offset", C.c_float * 3)]


class MarchParams(C.Structure):
    _fields_ = [("rays", C.c_uint32), ("second_bounce", C.c_uint32), ("max_steps", C.c_uint32), ("frame", C.c_uint32),
                ("step_size", C.c_float), ("normal_offset", C.c_float), ("shadow_bias", C.c_float),
                ("sky", C.c_float * 3), ("sky_scale", C.c_float), ("pad", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_uint32), ("max_batch_views", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("hbm_budget", C.c_uint64), ("cone", ConeParams),
                ("trace_variant", C.c_uint32), ("pad", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("flags", C.c_uint32), ("moves", C.POINTER(Move)), ("nmoves", C.c_uint32),
                ("nviews", C.c_uint32), ("views", C.POINTER(View))]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("batch", C.c_uint32), ("queued_ms", C.c_double), ("latency_ms", C.c_double),
                ("pixels", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("requests_cancelled", C.c_uint64), ("batches", C.c_uint64),
                ("pixels", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("mean_batch_views", C.c_double), ("hbm_used", C.c_uint64), ("hbm_budget", C.c_uint64),
                ("pending", C.c_uint32), ("inflight", C.c_uint32), ("trace_variant", C.c_uint32),
                ("trace_variants", C.c_uint32), ("trace_tile", C.c_uint32 * 2), ("trace_ctas_per_sm", C.c_uint32),
                ("pad", C.c_uint32), ("tune_ms", C.c_float * 8)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("flags", C.c_uint32), ("hbm_budget", C.c_uint64)]


class Scene(C.Structure):
    _fields_ = [("ntris", C.c_uint64), ("nobjects", C.c_uint32), ("pad", C.c_uint32),
                ("tri_xyz", C.POINTER(C.c_float)), ("albedo", C.POINTER(C.c_uint32)),
                ("roughness", C.POINTER(C.c_float)), ("object_first", C.POINTER(C.c_uint32)),
                ("object_count", C.POINTER(C.c_uint32)), ("bounds", Bounds), ("light", Light),
                ("eye", C.c_float * 3), ("target", C.c_float * 3)]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
F32 = C.c_float
PF = C.POINTER(C.c_float)

# name -> (restype, argtypes); every symbol of include/f184gi.h
PROTOTYPES = {
    "f184gi_last_error": (C.c_char_p, []),
    "f184gi_abi_version": (C.c_int, []),
    "f184gi_kernel_launches": (C.c_uint64, []),
    "f184gi_create": (C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    "f184gi_destroy": (C.c_int, [P]),
    "f184gi_memory_used": (C.c_int, [P, C.POINTER(U64)]),
    "f184gi_grid_create": (C.c_int, [P, C.POINTER(GridDesc), C.POINTER(U32)]),
    "f184gi_grid_destroy": (C.c_int, [P, U32]),
    "f184gi_grid_bytes": (C.c_int, [C.POINTER(GridDesc), C.POINTER(U64)]),
    "f184gi_voxelize": (C.c_int, [P, U32, P, P, U64, C.POINTER(Bounds), C.POINTER(Light), P, U32, P]),
    "f184gi_mip": (C.c_int, [P, U32, U32, U32, P]),
    "f184gi_trace": (C.c_int, [P, U32, C.POINTER(View), U32, C.POINTER(ConeParams), P]),
    "f184gi_selftest_bounded_wait": (C.c_int, [P, U32, U32, P]),
    "f184gi_trace_count": (C.c_int, [P, U32, C.POINTER(View), U32, C.POINTER(ConeParams), C.POINTER(C.c_uint64), P]),
    "f184gi_cone_params_default": (None, [C.POINTER(ConeParams)]),
    "f184gi_gbuffer": (C.c_int, [P, P, P, U64, C.POINTER(View), P, P]),
    "f184gi_march_params_default": (None, [C.POINTER(MarchParams)]),
    "f184gi_march": (C.c_int, [P, U32, C.POINTER(View), U32, C.POINTER(MarchParams), P]),
    "f184gi_blur": (C.c_int, [P, P, P, U32, U32, P, P]),
    "f184gi_gbuffer_static": (C.c_int, [P, P, P, U64, C.POINTER(View), P, P]),
    "f184gi_transform": (C.c_int, [P, P, U64, PF, P, P]),
    "f184gi_apply_moves": (C.c_int, [P, P, C.POINTER(Move), U32, U64, P]),
    "f184gi_sync": (C.c_int, [P, P]),
    "f184gi_grid_get_frame": (C.c_int, [P, U32, C.POINTER(GridFrame)]),
    "f184gi_frame_from_bounds": (C.c_int, [C.POINTER(Bounds), U32, PF, C.POINTER(GridFrame)]),
    "f184gi_grid_read_level": (C.c_int, [P, U32, U32, U32, P]),
    "f184gi_grid_read_shadow": (C.c_int, [P, U32, P]),
    "f184gi_grid_read_counts": (C.c_int, [P, U32, P]),
    "f184gi_grid_level_ptr": (C.c_int, [P, U32, U32, C.POINTER(P), C.POINTER(U64)]),
    "f184gi_camera_perspective": (None, [F32, F32, F32, F32, PF]),
    "f184gi_camera_ortho": (None, [F32, F32, F32, F32, PF]),
    "f184gi_camera_look_at": (None, [PF, PF, PF]),
    "f184gi_mat4_inverse": (C.c_int, [PF, PF]),
    "f184gi_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(P)]),
    "f184gi_server_destroy": (C.c_int, [P]),
    "f184gi_server_add_scene": (C.c_int, [P, U32, C.POINTER(GridDesc), P, P, U64, C.POINTER(Bounds), C.POINTER(Light)]),
    "f184gi_server_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(U64)]),
    "f184gi_server_wait": (C.c_int, [P, U64, U32, C.POINTER(RequestResult)]),
    "f184gi_server_cancel": (C.c_int, [P, U64]),
    "f184gi_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "f184gi_server_set_log": (C.c_int, [P, C.c_char_p]),
    "f184gi_server_submit_batch": (C.c_int, [P, C.POINTER(Request), U32, C.POINTER(U64)]),
    "f184gi_scene_generate": (C.c_int, [U64, U64, U32, C.POINTER(C.POINTER(Scene))]),
    "f184gi_scene_free": (None, [C.POINTER(Scene)]),
    "f184gi_scene_move_objects": (C.c_int, [C.POINTER(Scene), U64, F32, F32, C.POINTER(U32), C.POINTER(U32)]),
    "f184gi_scene_camera": (C.c_int, [C.POINTER(Scene), U64, U32, PF, PF]),
    "f184gi_gltf_load": (C.c_int, [C.c_char_p, C.POINTER(C.POINTER(Scene))]),
    "f184gi_reference_sun_direction": (None, [PF]),
}

_lib = None


def load():
    """Load libf184gi.so (built in-tree by final184_gb300.build); raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libf184gi.so is not built; run `python -m final184_gb300.build` "
                          "(the CUDA path has no fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class F184Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("f184gi error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != OK:
        raise F184Error(rc, load().f184gi_last_error().decode())
    return rc
