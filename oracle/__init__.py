"""Python wrapper of the CPU oracle (oracle.cpp).  TEST INFRASTRUCTURE ONLY.

Only the test suite, the smoke check and the benchmark's CPU-baseline leg import this package; the product
(final184_gb300) never does.  Structures are declared here independently of the product's bindings.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Bounds(C.Structure):
    _fields_ = [("min", Vec3), ("pad0", C.c_float), ("max", Vec3), ("pad1", C.c_float)]


class Light(C.Structure):
    _fields_ = [("luminance", C.c_float * 3), ("direction", C.c_float * 3)]


class GridFrame(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("voxel_size", C.c_double), ("inv_voxel_fixed", C.c_double),
                ("light_clip", C.c_double * 16), ("shadow_bias", C.c_double), ("light_dir", C.c_double * 3),
                ("light_vox", C.c_float * 12), ("shadow_bias_f", C.c_float), ("pad_f", C.c_float * 3)]


class ConeParams(C.Structure):
    _fields_ = [("diffuse_cones", C.c_uint32), ("diffuse_tan_half", C.c_float), ("diffuse_tilt_deg", C.c_float),
                ("step_factor", C.c_float), ("max_distance", C.c_float), ("alpha_stop", C.c_float),
                ("start_offset", C.c_float), ("min_spec_tan_half", C.c_float), ("specular", C.c_uint32),
                ("pad", C.c_uint32)]


def default_params():
    return ConeParams(5, 0.57735026918962576, 60.0, 0.5, 0.0, 1.0, 1.0, 0.05, 1, 0)


class MarchParams(C.Structure):
    _fields_ = [("rays", C.c_uint32), ("second_bounce", C.c_uint32), ("max_steps", C.c_uint32), ("frame", C.c_uint32),
                ("step_size", C.c_float), ("normal_offset", C.c_float), ("shadow_bias", C.c_float),
                ("sky", C.c_float * 3), ("sky_scale", C.c_float), ("pad", C.c_float)]


def default_march_params():
    """The reference's constants (indirect.frag:116,138,161,165,180; four rays with a second bounce)."""
    return MarchParams(4, 1, 60, 0, 0.2, 0.06, 0.005, (C.c_float * 3)(0.7, 0.8, 1.0), 0.4, 0.0)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = C.CDLL(path)
        V = C.c_void_p
        _lib.orc_grid_frame.argtypes = [C.POINTER(Bounds), C.c_uint32, V, C.POINTER(GridFrame)]
        _lib.orc_raster.argtypes = [V, C.c_uint32, C.c_uint32, V, C.c_uint64, V, C.c_int]
        _lib.orc_gbuffer_resolve.argtypes = [V, C.c_uint32, C.c_uint32, V, V, V, V, V, V, V]
        for n in ("orc_voxelize_f64", "orc_voxelize_f32"):
            getattr(_lib, n).argtypes = [C.POINTER(GridFrame), C.c_uint32, C.c_uint32, V, V, C.c_uint64,
                                         C.POINTER(Light), V, V, V, C.c_int]
        _lib.orc_shade.argtypes = [C.POINTER(GridFrame), C.c_uint32, V, V, C.c_uint64, V]
        for n in ("orc_mip_f64", "orc_mip_f32", "orc_mip_aniso_f64"):
            getattr(_lib, n).argtypes = [V, C.c_uint32, C.c_uint32, C.c_int]
        for n in ("orc_trace_f64", "orc_trace_f32"):
            getattr(_lib, n).argtypes = [C.POINTER(GridFrame), C.c_uint32, C.c_uint32, C.c_uint32, V, V, V,
                                         C.c_uint32, C.c_uint32, V, V, V, C.POINTER(ConeParams), V, C.c_uint32,
                                         C.c_uint32, C.c_int]
        _lib.orc_trace_count_f32.argtypes = [C.POINTER(GridFrame), C.c_uint32, C.c_uint32, C.c_uint32, V, V, V,
                                             C.c_uint32, C.c_uint32, V, V, V, C.POINTER(ConeParams), V, C.c_uint32,
                                             C.c_uint32, C.c_int, V]
        _lib.orc_cone_f64.argtypes = [V, C.c_uint32, C.c_uint32, C.c_uint32, V, V, C.c_double,
                                      C.POINTER(ConeParams), V]
        _lib.orc_make_coord_space.argtypes = [V, V]
        _lib.orc_refvox.argtypes = [C.POINTER(GridFrame), C.c_uint32, V, V, C.c_uint64, V]
        for n in ("orc_march_f32", "orc_march_f64"):
            getattr(_lib, n).argtypes = [C.POINTER(GridFrame), C.c_uint32, V, V, C.c_uint32, C.POINTER(Light), V, V,
                                         C.c_uint32, C.c_uint32, V, V, C.POINTER(MarchParams), V, C.c_uint32,
                                         C.c_uint32, C.c_int]
        _lib.orc_sincos_turns.argtypes = [C.c_float, V, V]
        for n in ("orc_blur_f32", "orc_blur_f64"):
            getattr(_lib, n).argtypes = [V, V, C.c_uint32, C.c_uint32, V]
        _lib.orc_exp2_poly.argtypes = [C.c_float]
        _lib.orc_exp2_poly.restype = C.c_float
        _lib.orc_pack_color565.argtypes = [V]
        _lib.orc_pack_color565.restype = C.c_uint32
        _lib.orc_pack_normal565.argtypes = [V]
        _lib.orc_pack_normal565.restype = C.c_uint32
        _lib.orc_unpack_color565.argtypes = [C.c_uint32, V]
        _lib.orc_unpack_normal565.argtypes = [C.c_uint32, V]
        _lib.orc_dominant_axis.argtypes = [V, V, V]
        _lib.orc_hemisphere_sample_cos.argtypes = [C.c_double, C.c_double, V]
        _lib.orc_oct_encode.argtypes = [V]
        _lib.orc_oct_encode.restype = C.c_uint32
        _lib.orc_oct_decode.argtypes = [C.c_uint32, V]
        _lib.orc_float_to_half.argtypes = [C.c_double]
        _lib.orc_float_to_half.restype = C.c_uint16
        _lib.orc_half_to_float.argtypes = [C.c_uint16]
        _lib.orc_half_to_float.restype = C.c_double
    return _lib


def ref_lib():
    """The reference's own Math + CCamera compiled from source (None when not built here)."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        try:
            _build.build_ref()  # rebuilt when ref_shim.cpp changed; a no-op where the reference tree is absent
        except RuntimeError:
            return None
        if not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
        V = C.c_void_p
        F = C.c_float
        _ref.ref_sizeof.argtypes = [C.c_int]
        _ref.ref_calc_perspective.argtypes = [F, F, F, F, V]
        _ref.ref_calc_ortho.argtypes = [F, F, F, F, V]
        _ref.ref_matrix4_inverse.argtypes = [V, V]
        _ref.ref_bbox_transformed.argtypes = [V, V, V, V]
        _ref.ref_frustum_box.argtypes = [V, V, V]
        _ref.ref_quat_euler_rotate.argtypes = [F, F, F, V, V]
        _ref.ref_matrix_trs.argtypes = [V, V, V, V]
        _ref.ref_frustum_define.argtypes = [V, V]
        _ref.ref_frustum_transformed.argtypes = [V, V, V]
        _ref.ref_frustum_inside_fast.argtypes = [V, V, V]
    return _ref


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def make_bounds(mn, mx):
    b = Bounds()
    b.min.x, b.min.y, b.min.z = (float(v) for v in mn)
    b.max.x, b.max.y, b.max.z = (float(v) for v in mx)
    return b


def make_light(lum, direction):
    lt = Light()
    for i in range(3):
        lt.luminance[i] = float(lum[i])
        lt.direction[i] = float(direction[i])
    return lt


def grid_frame(bounds, dim, light_dir):
    f = GridFrame()
    d = np.asarray(light_dir, dtype=np.float32)
    rc = lib().orc_grid_frame(C.byref(bounds), dim, _p(d), C.byref(f))
    assert rc == 0
    return f


def frame_matrix(f):
    return np.array(f.light_clip, dtype=np.float64).reshape(4, 4)


def raster(M, width, height, tri, nthreads=0):
    M = np.ascontiguousarray(M, dtype=np.float64).ravel()
    tri = np.ascontiguousarray(tri, dtype=np.float32).ravel()
    keys = np.empty(width * height, dtype=np.uint64)
    assert lib().orc_raster(_p(M), width, height, _p(tri), tri.size // 9, _p(keys), nthreads) == 0
    return keys.reshape(height, width)


def shadow_depth(keys):
    """keys -> FP32 depth, 1.0 where empty."""
    k = keys.ravel()
    d = (k >> np.uint64(32)).astype(np.uint32).view(np.float32).copy()
    d[k == np.uint64(0xFFFFFFFFFFFFFFFF)] = 1.0
    return d.reshape(keys.shape)


def gbuffer_resolve(keys, tri, rough, view):
    h, w = keys.shape
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    tri = np.ascontiguousarray(tri, dtype=np.float32).ravel()
    rough = np.ascontiguousarray(rough, dtype=np.float32)
    view = np.ascontiguousarray(view, dtype=np.float32).ravel()
    depth = np.empty(w * h, np.float32)
    normal = np.empty(w * h, np.uint32)
    r = np.empty(w * h, np.uint16)
    t = np.empty(w * h, np.uint32)
    assert lib().orc_gbuffer_resolve(_p(keys), w, h, _p(tri), _p(rough), _p(view), _p(depth), _p(normal), _p(r),
                                     _p(t)) == 0
    return depth.reshape(h, w), normal.reshape(h, w), r.reshape(h, w), t.reshape(h, w)


def voxelize(frame, dim, shadow_res, tri, albedo, light, shadow, f64=True, nthreads=0):
    tri = np.ascontiguousarray(tri, dtype=np.float32).ravel()
    albedo = np.ascontiguousarray(albedo, dtype=np.uint32)
    shadow = np.ascontiguousarray(shadow, dtype=np.float32)
    dt = np.float64 if f64 else np.float32
    rgba = np.empty(dim ** 3 * 4, dtype=dt)
    counts = np.empty(dim ** 3, dtype=np.uint32)
    fn = lib().orc_voxelize_f64 if f64 else lib().orc_voxelize_f32
    assert fn(C.byref(frame), dim, shadow_res, _p(tri), _p(albedo), tri.size // 9, C.byref(light), _p(shadow),
              _p(rgba), _p(counts), nthreads) == 0
    return rgba.reshape(dim, dim, dim, 4), counts.reshape(dim, dim, dim)


def shade(frame, shadow_res, shadow, ijk):
    ijk = np.ascontiguousarray(ijk, dtype=np.uint32)
    shadow = np.ascontiguousarray(shadow, dtype=np.float32)
    out = np.empty(ijk.shape[0], dtype=np.uint8)
    assert lib().orc_shade(C.byref(frame), shadow_res, _p(shadow), _p(ijk), ijk.shape[0], _p(out)) == 0
    return out


def chain_size(dim, levels, aniso=False):
    n = 0
    for l in range(levels):
        d = dim >> l
        n += d ** 3 * 4 * (6 if (aniso and l > 0) else 1)
    return n


def mip(l0, levels, f64=True, aniso=False, nthreads=0):
    """Returns the packed chain (flat) and a list of per-level views [(d,d,d,4)] (aniso: (6,d,d,d,4) for l>0)."""
    dim = l0.shape[0]
    dt = np.float64 if f64 else np.float32
    chain = np.zeros(chain_size(dim, levels, aniso), dtype=dt)
    chain[: dim ** 3 * 4] = np.asarray(l0, dtype=dt).ravel()
    if aniso:
        assert f64
        assert lib().orc_mip_aniso_f64(_p(chain), dim, levels, nthreads) == 0
    else:
        fn = lib().orc_mip_f64 if f64 else lib().orc_mip_f32
        assert fn(_p(chain), dim, levels, nthreads) == 0
    views = []
    off = 0
    for l in range(levels):
        d = dim >> l
        k = 6 if (aniso and l > 0) else 1
        n = d ** 3 * 4 * k
        v = chain[off: off + n]
        views.append(v.reshape(6, d, d, d, 4) if k == 6 else v.reshape(d, d, d, 4))
        off += n
    return chain, views


def trace(frame, dim, levels, chain, view, proj, width, height, depth, normal, rough, params=None, rows=None,
          f64=True, aniso=False, nthreads=0):
    dt = np.float64 if f64 else np.float32
    chain = np.ascontiguousarray(chain, dtype=dt)
    view = np.ascontiguousarray(view, dtype=np.float32).ravel()
    proj = np.ascontiguousarray(proj, dtype=np.float32).ravel()
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    normal = np.ascontiguousarray(normal, dtype=np.uint32)
    rough = np.ascontiguousarray(rough, dtype=np.uint16)
    out = np.zeros(2 * width * height * 4, dtype=dt)
    r0, r1 = rows if rows is not None else (0, height)
    fn = lib().orc_trace_f64 if f64 else lib().orc_trace_f32
    p = params if params is not None else default_params()
    assert fn(C.byref(frame), dim, levels, 1 if aniso else 0, _p(chain), _p(view), _p(proj), width, height,
              _p(depth), _p(normal), _p(rough), C.byref(p), _p(out), r0, r1, nthreads) == 0
    return out.reshape(2, height, width, 4)


def trace_count(frame, dim, levels, chain, view, proj, width, height, depth, normal, rough, params=None,
                aniso=False, nthreads=0):
    """FP32 trace of the whole image plus its totals: (out, cone steps, level samples)."""
    chain = np.ascontiguousarray(chain, dtype=np.float32)
    view = np.ascontiguousarray(view, dtype=np.float32).ravel()
    proj = np.ascontiguousarray(proj, dtype=np.float32).ravel()
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    normal = np.ascontiguousarray(normal, dtype=np.uint32)
    rough = np.ascontiguousarray(rough, dtype=np.uint16)
    out = np.zeros(2 * width * height * 4, dtype=np.float32)
    counts = np.zeros(2, dtype=np.uint64)
    p = params if params is not None else default_params()
    assert lib().orc_trace_count_f32(C.byref(frame), dim, levels, 1 if aniso else 0, _p(chain), _p(view), _p(proj),
                                     width, height, _p(depth), _p(normal), _p(rough), C.byref(p), _p(out), 0, height,
                                     nthreads, _p(counts)) == 0
    return out.reshape(2, height, width, 4), int(counts[0]), int(counts[1])


def cone(chain, dim, levels, origin, direction, tan_half, params=None, aniso=False):
    chain = np.ascontiguousarray(chain, dtype=np.float64)
    o = np.ascontiguousarray(origin, dtype=np.float64)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    out = np.zeros(4, dtype=np.float64)
    p = params if params is not None else default_params()
    assert lib().orc_cone_f64(_p(chain), dim, levels, 1 if aniso else 0, _p(o), _p(d), tan_half, C.byref(p),
                              _p(out)) == 0
    return out


def make_coord_space(n):
    n = np.ascontiguousarray(n, dtype=np.float64)
    out = np.zeros(9, dtype=np.float64)
    lib().orc_make_coord_space(_p(n), _p(out))
    return out.reshape(3, 3)  # rows: x, y, z axes


def refvox(frame, dim, tri, albedo):
    """The reference's voxel volume: (dim, dim, dim) uint32 = RGB565 albedo | 565 normal << 16, x fastest."""
    tri = np.ascontiguousarray(tri, dtype=np.float32).ravel()
    albedo = np.ascontiguousarray(albedo, dtype=np.uint32).ravel()
    vol = np.empty(dim ** 3, dtype=np.uint32)
    assert lib().orc_refvox(C.byref(frame), dim, _p(tri), _p(albedo), tri.size // 9, _p(vol)) == 0
    return vol.reshape(dim, dim, dim)


def march(frame, dim, vol, shadow, light, view, proj, width, height, depth, normal, params=None, rows=None,
          f64=False, nthreads=0):
    """The reference-faithful march: (height, width, 4) [indirect.rgb, view distance].  FP32 = the device's
    operation sequence; FP64 = the same method in double."""
    vol = np.ascontiguousarray(vol, dtype=np.uint32)
    shadow = np.ascontiguousarray(shadow, dtype=np.float32)
    res = shadow.shape[0]
    view = np.ascontiguousarray(view, dtype=np.float32).ravel()
    proj = np.ascontiguousarray(proj, dtype=np.float32).ravel()
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    normal = np.ascontiguousarray(normal, dtype=np.uint32)
    out = np.zeros(width * height * 4, dtype=np.float64 if f64 else np.float32)
    r0, r1 = rows if rows is not None else (0, height)
    p = params if params is not None else default_march_params()
    fn = lib().orc_march_f64 if f64 else lib().orc_march_f32
    assert fn(C.byref(frame), dim, _p(vol), _p(shadow), res, C.byref(light), _p(view), _p(proj), width, height,
              _p(depth), _p(normal), C.byref(p), _p(out), r0, r1, nthreads) == 0
    return out.reshape(height, width, 4)


def sincos_turns(v):
    s, c = np.zeros(1, np.float32), np.zeros(1, np.float32)
    lib().orc_sincos_turns(float(v), _p(s), _p(c))
    return float(s[0]), float(c[0])


def blur(img, depth, f64=False):
    """The reference's two blur passes: img (H, W, 4), depth (H, W) -> (H, W, 4) with alpha 0."""
    dt = np.float64 if f64 else np.float32
    img = np.ascontiguousarray(img, dtype=dt)
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    H, W = depth.shape
    out = np.empty((H, W, 4), dtype=dt)
    fn = lib().orc_blur_f64 if f64 else lib().orc_blur_f32
    assert fn(_p(img), _p(depth), W, H, _p(out)) == 0
    return out


def exp2_poly(t):
    return float(lib().orc_exp2_poly(float(t)))
