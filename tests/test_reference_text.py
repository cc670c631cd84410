"""The oracle against the reference's own shader text (CPU).

oracle/glsl_pin.py takes the reference's shader functions out of its sources verbatim (Shader/math.inc,
Shader/Lighting/indirect.frag, Pipelang/Internal/main.lua) and compiles them as C++ under a small GLSL vocabulary,
so the restatement the oracle, the CUDA kernels and the FP32 CPU baseline share is checked against the reference's
text itself, not against hand-written known answers:
  - the 565 packing (main.lua:269-270) and the dominant axis (main.lua:100-115): bit-identical;
  - unpackColor565 over all 2^16 codes: bit-identical to the oracle rounded to FP32; unpackNormal565,
    make_coord_space and hemisphereSample_cos (indirect.frag:71-102, math.inc:76-81): within FP32 rounding;
  - getIndirect and main()'s combine of four rays with their second bounces (indirect.frag:104-222, the temporal
    blend excluded) on 20k surface points of a seeded scene against the oracle's FP32 march
    (orc_march_points_f32, the sequence the device's march kernel runs bit for bit), fed the same volume, shadow
    map, light and random numbers.
Skipped where the reference sources are absent (they are not on GPU machines).
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import glsl_pin


@pytest.fixture(scope="module")
def glsl(orc):
    if not os.path.isdir(glsl_pin.REF_ROOT):
        pytest.skip("reference sources absent")
    lib = C.CDLL(glsl_pin.build())
    V = C.c_void_p
    lib.ref_hemisphere_sample_cos.argtypes = [C.c_float, C.c_float, V]
    lib.ref_make_coord_space.argtypes = [V, V]
    lib.ref_unpack_color565.argtypes = [C.c_uint32, V]
    lib.ref_unpack_normal565.argtypes = [C.c_uint32, V]
    lib.ref_dominant_axis.argtypes = [V]
    lib.ref_dominant_axis.restype = C.c_uint32
    lib.ref_pack565.argtypes = [V, V, V]
    lib.ref_march_setup.argtypes = [V, C.c_int, V, C.c_int, V, V, V, V, V, V, C.c_uint32]
    lib.ref_march_points.argtypes = [V, V, V, C.c_uint64, V]
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_pack565_and_dominant_axis_bit_identical(glsl, orc):
    rng = np.random.default_rng(1)
    o = orc.lib()
    for _ in range(3000):
        rgba = rng.uniform(0, 1, 4).astype(np.float32)
        n = rng.uniform(-1, 1, 3).astype(np.float32)
        got = np.zeros(2, np.uint32)
        glsl.ref_pack565(_p(rgba), _p(n), _p(got))
        assert got[0] == o.orc_pack_color565(_p(rgba[:3].copy()))
        assert got[1] == o.orc_pack_normal565(_p(n))
    for k in range(5000):
        v = rng.normal(size=9).astype(np.float32)
        if k % 5 == 0:  # axis-aligned faces and ties between components
            v = np.round(v).astype(np.float32)
        want = o.orc_dominant_axis(_p(v[0:3].copy()), _p(v[3:6].copy()), _p(v[6:9].copy()))
        assert glsl.ref_dominant_axis(_p(v)) == want


def test_unpack565_coord_space_and_cosine_sampling(glsl, orc):
    o = orc.lib()
    got, want = np.zeros(3, np.float32), np.zeros(3, np.float64)
    for x in range(1 << 16):
        glsl.ref_unpack_color565(x, _p(got))
        o.orc_unpack_color565(x, _p(want))
        assert np.array_equal(got, want.astype(np.float32)), x
    for x in range(0, 1 << 16, 7):
        glsl.ref_unpack_normal565(x, _p(got))
        o.orc_unpack_normal565(x, _p(want))
        assert np.abs(got - want).max() < 4e-7, x
    rng = np.random.default_rng(2)
    m32, m64 = np.zeros(9, np.float32), np.zeros(9, np.float64)
    for _ in range(5000):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        n32 = n.astype(np.float32)
        glsl.ref_make_coord_space(_p(n32), _p(m32))
        o.orc_make_coord_space(_p(n32.astype(np.float64)), _p(m64))
        assert np.abs(m32 - m64).max() < 2e-6
    for _ in range(5000):
        u, v = (float(np.float32(x)) for x in rng.uniform(0, 1, 2))
        glsl.ref_hemisphere_sample_cos(u, v, _p(got))
        o.orc_hemisphere_sample_cos(u, v, _p(want))
        # FP32 conditioning of the reference's sqrt(1 - cos^2): an ulp of 1 - cos^2 moves sin by ~6e-8 / sin
        st = np.sqrt(1.0 - (1.0 - u))
        assert np.abs(got - want).max() < 1e-6 + 3e-7 / max(st, 1e-4), (u, v)


def test_march_against_reference_getindirect(glsl, orc):
    """The reference's getIndirect + four-ray combine, compiled from its text, against the oracle's FP32 march on
    20k points.  The world -> voxel map is a power-of-two frame (origin -8 m, 1/8 m voxels, the reference's 128^3
    volume) written as the reference's VoxelProj (x, y: * 0.5 + 0.5, then * 128) so both sides round identically;
    the shadow transform is the light frame's rows as ShadowProj with ShadowView = identity."""
    import final184_gb300 as g

    dim, res = 128, 2048
    sc = g.SyntheticScene(184, 20000, 200)
    tri_xyz = (sc.tri_xyz * np.float32(0.75)).astype(np.float32)  # the room ([-7.5, 7.5] m) inside the grid
    ld = np.array(sc.light.direction, np.float32)
    fo = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), dim, ld)
    for a in range(3):
        fo.origin[a] = -8.0
    fo.voxel_size, fo.inv_voxel_fixed = 0.125, 2048.0
    vol = orc.refvox(fo, dim, tri_xyz, sc.albedo).astype(np.uint32)
    assert (vol != 0).mean() > 0.01
    shadow = np.ascontiguousarray(orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, tri_xyz)),
                                  dtype=np.float32)
    voxel_proj = np.array([[0.125, 0, 0, 0], [0, 0.125, 0, 0], [0, 0, 0.0625, 0.5], [0, 0, 0, 1]], np.float32)
    ident = np.eye(4, dtype=np.float32)
    shadow_proj = orc.frame_matrix(fo).astype(np.float32)
    lum = np.array(sc.light.luminance, np.float32)
    glsl.ref_march_setup(_p(vol), dim, _p(shadow), res, _p(voxel_proj), _p(ident), _p(shadow_proj), _p(ident),
                         _p(lum), _p(ld), 0)
    # surface points: random points on random triangles inside the grid, face normals facing the room's centre
    rng = np.random.default_rng(3)
    tri = tri_xyz.reshape(-1, 3, 3).astype(np.float64)
    pick = rng.integers(0, len(tri), 60000)
    b = rng.uniform(0, 1, (len(pick), 2))
    flip = b.sum(1) > 1
    b[flip] = 1 - b[flip]
    t = tri[pick]
    p = t[:, 0] + b[:, :1] * (t[:, 1] - t[:, 0]) + b[:, 1:] * (t[:, 2] - t[:, 0])
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    ln = np.linalg.norm(n, axis=1)
    keep = (ln > 1e-9) & (np.abs(p).max(1) < 7.4)
    p, n, ln = p[keep][:20000], n[keep][:20000], ln[keep][:20000]
    n = n / ln[:, None]
    n[(n * p).sum(1) > 0] *= -1
    wpos = np.ascontiguousarray(p, np.float32)
    wnorm = np.ascontiguousarray(n, np.float32)
    pix = np.arange(len(wpos), dtype=np.uint32) * np.uint32(2654435761)
    rands = np.zeros((len(wpos), 8, 2), np.float32)
    o = orc.lib()
    o.orc_march_rands.argtypes = [C.c_uint32, C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p]
    o.orc_march_rands(0, _p(pix), len(pix), 8, _p(rands))
    want = np.zeros((len(wpos), 3), np.float32)
    o.orc_march_points_f32.argtypes = [C.POINTER(orc.GridFrame), C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                       C.POINTER(orc.Light), C.POINTER(orc.MarchParams), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_uint64, C.c_void_p]
    light = orc.make_light(list(lum), list(ld))
    params = orc.default_march_params()
    assert o.orc_march_points_f32(C.byref(fo), dim, _p(vol), _p(shadow), res, C.byref(light), C.byref(params),
                                  _p(pix), _p(wpos), _p(wnorm), len(wpos), _p(want)) == 0
    got = np.zeros_like(want)
    glsl.ref_march_points(_p(wpos), _p(wnorm), _p(rands), len(wpos), _p(got))
    same = np.all(got.view(np.uint32) == want.view(np.uint32), axis=1)
    rel = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want.astype(np.float64)), 1e-30)
    close = np.all((rel < 1e-3) | (np.abs(got - want) == 0), axis=1)
    lit = (want > 0).any(1).mean()
    print("reference getIndirect vs FP32 march: %d points, %.2f%% lit, %.3f%% bit-identical, %.3f%% within 1e-3, "
          "%d apart" % (len(wpos), 100 * lit, 100 * same.mean(), 100 * close.mean(), int((~close).sum())))
    assert lit > 0.2
    assert close.mean() > 0.999
    assert same.mean() > 0.7
