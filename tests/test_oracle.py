"""Known-answer tests that pin the CPU oracle (no GPU).

The reference has no tests, fixtures or golden vectors for this path, and its GLSL cannot run here; these
known answers are derived by hand or by an independent exact (integer / Python) restatement:
  - the reference's shader helpers restated in the oracle (565 packing, make_coord_space, dominant axis,
    hemisphereSample_cos) against hand-computed values,
  - the exact raster against hand-counted coverage,
  - conservative voxelization against a pure-Python big-integer separating-axis test,
  - a uniformly lit floor (analytic injected radiance) and an occluder (analytic shadow),
  - a constant-density grid (analytic cone transmittance 1 - (1 - a)^n),
  - order independence of voxelization.
"""
import ctypes as C
import math

import numpy as np
import pytest


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ---------------- reference shader helpers ----------------

def test_pack_color565_kat(orc):
    lib = orc.lib()
    assert lib.orc_pack_color565(_p(np.array([1, 1, 1], np.float32))) == 0xFFFF
    assert lib.orc_pack_color565(_p(np.array([0, 0, 0], np.float32))) == 0
    # uint(0.5 * 31) = 15, uint(0.5 * 63) = 31 (truncation, main.lua:269)
    assert lib.orc_pack_color565(_p(np.array([0.5, 0.5, 0.5], np.float32))) == (15 << 11) | (31 << 5) | 15
    out = np.zeros(3)
    lib.orc_unpack_color565(0xFFFF, _p(out))
    assert np.allclose(out, 1.0)
    lib.orc_unpack_color565((31 << 11), _p(out))
    assert np.allclose(out, [1, 0, 0])


def test_pack_normal565_kat(orc):
    lib = orc.lib()
    # main.lua:270: (n.r*16+15) << 11 | (n.g*32+31) << 5 | (n.b*16+15)
    assert lib.orc_pack_normal565(_p(np.array([0, 0, 0], np.float32))) == (15 << 11) | (31 << 5) | 15
    assert lib.orc_pack_normal565(_p(np.array([1, 1, 1], np.float32))) == (31 << 11) | (63 << 5) | 31
    out = np.zeros(3)
    # indirect.frag:96-102 reads x from the LOW five bits although the pack stored r in the high bits;
    # the restatement keeps that channel order
    lib.orc_unpack_normal565(31, _p(out))  # low field = 31 -> x = 31/16 - 1 = 0.9375 ; y, z = -1
    want = np.array([0.9375, -1.0, -1.0])
    assert np.allclose(out, want / np.linalg.norm(want))


def test_make_coord_space_kat(orc):
    f = orc.make_coord_space([0.0, 0.0, 1.0])
    # h = (1, 0, 1): y = normalize(h x z) = (0, -1, 0), x = z x y = (1, 0, 0)
    assert np.allclose(f[0], [1, 0, 0]) and np.allclose(f[1], [0, -1, 0]) and np.allclose(f[2], [0, 0, 1])
    rng = np.random.default_rng(1)
    for _ in range(200):
        n = rng.normal(size=3)
        f = orc.make_coord_space(n)
        assert np.allclose(f @ f.T, np.eye(3), atol=1e-12)
        assert np.allclose(f[2], n / np.linalg.norm(n))


def test_dominant_axis_kat(orc):
    lib = orc.lib()

    def dom(a, b, c):
        return lib.orc_dominant_axis(_p(np.array(a, np.float32)), _p(np.array(b, np.float32)),
                                     _p(np.array(c, np.float32)))

    assert dom([0, 0, 0], [1, 0, 0], [0, 1, 0]) == 0  # normal along z -> Z (main.lua:108-114)
    assert dom([0, 0, 0], [0, 1, 0], [0, 0, 1]) == 1  # normal along x -> X
    assert dom([0, 0, 0], [1, 0, 0], [0, 0, 1]) == 2  # normal along y -> Y
    assert dom([0, 0, 0], [0, 0, 1], [1, -1, 0]) == 2  # |n.x| == |n.y| > n.z: ties go to Y
    assert dom([0, 0, 0], [1, 0, -1], [0, 1, 0]) == 0  # |n.x| == |n.z|: ties go to Z


def test_hemisphere_sample_cos_kat(orc):
    lib = orc.lib()
    out = np.zeros(3)
    lib.orc_hemisphere_sample_cos(0.0, 0.0, _p(out))
    assert np.allclose(out, [0, 0, 1])
    lib.orc_hemisphere_sample_cos(1.0, 0.25, _p(out))
    assert np.allclose(out, [0, 1, 0], atol=1e-7)
    lib.orc_hemisphere_sample_cos(0.75, 0.5, _p(out))  # cos(theta) = 0.5
    assert np.isclose(out[2], 0.5) and np.isclose(np.linalg.norm(out), 1.0)


def test_half_conversion_matches_ieee(orc):
    lib = orc.lib()
    rng = np.random.default_rng(2)
    xs = np.concatenate([rng.normal(size=4000) * 10.0 ** rng.integers(-8, 5, 4000),
                         [0.0, -0.0, 65504.0, 65519.9, 65520.0, 6e-8, 2.0 ** -25, 1.0 + 2.0 ** -11]])
    with np.errstate(over="ignore"):  # values past 65520 round to infinity on purpose
        for x in xs:
            h = lib.orc_float_to_half(float(x))
            assert h == int(np.array([x], np.float64).astype(np.float16).view(np.uint16)[0]), x
            if not math.isinf(np.float16(x)):
                assert lib.orc_half_to_float(h) == float(np.float16(x))


def test_oct_codec_round_trip(orc):
    lib = orc.lib()
    rng = np.random.default_rng(3)
    out = np.zeros(3)
    for _ in range(2000):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        code = lib.orc_oct_encode(_p(n))
        lib.orc_oct_decode(code, _p(out))
        assert np.dot(out, n) > math.cos(2e-3)


# ---------------- exact raster ----------------

def test_raster_half_viewport_triangle(orc):
    M = np.eye(4)
    tri = np.array([-1, -1, 0.5, 1, -1, 0.5, -1, 1, 0.5], np.float32)
    keys = orc.raster(M, 8, 8, tri)
    cov = keys != np.uint64(0xFFFFFFFFFFFFFFFF)
    py, px = np.nonzero(cov)
    assert set(zip(px, py)) == {(x, y) for x in range(8) for y in range(8) if x + y <= 7}  # inclusive edges
    d = orc.shadow_depth(keys)
    assert np.all(d[cov] == np.float32(0.5))
    assert np.all((keys[cov] & np.uint64(0xffffffff)) == 0)


def test_raster_nearest_wins_and_ties_to_lowest_index(orc):
    M = np.eye(4)
    full = [-1, -1, 0.5, 3, -1, 0.5, -1, 3, 0.5]
    near = [-1, -1, 0.25, 3, -1, 0.25, -1, 3, 0.25]
    keys = orc.raster(M, 4, 4, np.array(full + near + full, np.float32))
    assert np.all((keys & np.uint64(0xffffffff)) == 1)
    keys = orc.raster(M, 4, 4, np.array(full + full, np.float32))
    assert np.all((keys & np.uint64(0xffffffff)) == 0)


def test_raster_clips_behind_near_plane(orc):
    M = np.eye(4)
    # z runs from -0.5 at x = -1 to 0.5 at x = 1: the half with z < 0 is clipped away (Vulkan 0 <= z <= w)
    tri = np.array([-1, -1, -0.5, 1, -1, 0.5, -1, 3, -0.5, 1, 3, 0.5, 1, -1, 0.5, -1, 3, -0.5], np.float32)
    keys = orc.raster(M, 8, 8, tri)
    cov = keys != np.uint64(0xFFFFFFFFFFFFFFFF)
    assert cov[:, 4:].all() and not cov[:, :4].any()
    d = orc.shadow_depth(keys)
    assert np.all(d[cov] >= 0) and np.allclose(d[0, 4:], 0.5 * ((np.arange(4, 8) + 0.5) / 8 * 2 - 1), atol=1e-6)


# ---------------- conservative voxelization ----------------

def _unit_frame(orc, dim):
    f = orc.grid_frame(orc.make_bounds((0, 0, 0), (dim, dim, dim)), dim, [0.0, -1.0, 0.0])
    # replace the placement with origin 0, voxel size 1 (the light part is unused when every texel is empty)
    for a in range(3):
        f.origin[a] = 0.0
    f.voxel_size = 1.0
    f.inv_voxel_fixed = 256.0
    return f


def _py_overlap(q, i, j, k):
    """Independent exact SAT in Python integers: triangle q (3x3 ints, 1/256 voxel) vs voxel box (i, j, k)."""
    c = (256 * i + 128, 256 * j + 128, 256 * k + 128)
    v = [[q[a][b] - c[b] for b in range(3)] for a in range(3)]
    h = 128
    for b in range(3):
        if min(x[b] for x in v) > h or max(x[b] for x in v) < -h:
            return False
    e = [[v[(t + 1) % 3][b] - v[t][b] for b in range(3)] for t in range(3)]
    n = [e[0][1] * (v[2][2] - v[0][2]) - e[0][2] * (v[2][1] - v[0][1]),
         e[0][2] * (v[2][0] - v[0][0]) - e[0][0] * (v[2][2] - v[0][2]),
         e[0][0] * (v[2][1] - v[0][1]) - e[0][1] * (v[2][0] - v[0][0])]
    if abs(sum(n[b] * v[0][b] for b in range(3))) > h * sum(abs(x) for x in n):
        return False
    for ed in e:
        for ax in range(3):
            u = [0, 0, 0]
            u[ax] = 1
            a = [ed[1] * u[2] - ed[2] * u[1], ed[2] * u[0] - ed[0] * u[2], ed[0] * u[1] - ed[1] * u[0]]
            p = [sum(a[b] * x[b] for b in range(3)) for x in v]
            r = h * sum(abs(x) for x in a)
            if min(p) > r or max(p) < -r:
                return False
    return True


def _py_voxels(tri, dim):
    q = [[round(float(np.float64(tri[3 * a + b]) * 256.0)) for b in range(3)] for a in range(3)]
    out = set()
    for k in range(dim):
        for j in range(dim):
            for i in range(dim):
                if _py_overlap(q, i, j, k):
                    out.add((i, j, k))
    return out


def _oracle_voxels(orc, tris, dim):
    f = _unit_frame(orc, dim)
    res = 64
    shadow = np.ones(res * res, np.float32)
    n = len(tris) // 9
    light = orc.make_light([1, 1, 1], [0, -1, 0])
    rgba, cnt = orc.voxelize(f, dim, res, np.array(tris, np.float32), np.full(n, 0xffffffff, np.uint32), light,
                             shadow)
    return cnt


def test_voxelize_hand_built_triangle(orc):
    # right triangle in the plane z = 2.5 (voxel centres of layer 2): legs from (0.5, 0.5) to 3.5
    tri = [0.5, 0.5, 2.5, 3.5, 0.5, 2.5, 0.5, 3.5, 2.5]
    cnt = _oracle_voxels(orc, tri, 8)
    got = {(i, j, k) for k, j, i in zip(*np.nonzero(cnt))}
    want = {(i, j, 2) for i in range(4) for j in range(4) if max(i, 0.5) + max(j, 0.5) <= 4}
    assert got == want
    assert (3, 1, 2) in got and (2, 2, 2) in got and (3, 2, 2) not in got  # corner touches count


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_voxelize_triangle_per_dominant_axis_matches_exact_python(orc, axis):
    rng = np.random.default_rng(10 + axis)
    for _ in range(4):
        base = rng.uniform(1.0, 7.0, size=(3, 3))
        base[:, axis] = rng.uniform(3.0, 3.6) + rng.uniform(-0.4, 0.4, 3)  # nearly perpendicular to `axis`
        tri = base.astype(np.float32).ravel()
        cnt = _oracle_voxels(orc, list(tri), 8)
        got = {(i, j, k) for k, j, i in zip(*np.nonzero(cnt))}
        assert got == _py_voxels(tri, 8)


def test_voxelize_random_triangles_match_exact_python(orc):
    rng = np.random.default_rng(5)
    tri = rng.uniform(0.0, 8.0, size=(6, 9)).astype(np.float32)
    tri[0, 2::3] = 4.0  # exactly on a voxel boundary plane: closed boxes on both sides count
    tri[1, 0::3] = 2.5
    for t in tri:
        cnt = _oracle_voxels(orc, list(t), 8)
        got = {(i, j, k) for k, j, i in zip(*np.nonzero(cnt))}
        assert got == _py_voxels(t, 8)


def _floor_scene(albedo_byte=255, occluder=False):
    tri = [-8, 0, -8, 8, 0, -8, 8, 0, 8, -8, 0, -8, 8, 0, 8, -8, 0, 8]
    if occluder:  # a roof over x in [-8, 0] at y = 5
        tri += [-8, 5, -8, 0, 5, -8, 0, 5, 8, -8, 5, -8, 0, 5, 8, -8, 5, 8]
    n = len(tri) // 9
    a = albedo_byte
    return np.array(tri, np.float32), np.full(n, 0xff000000 | (a << 16) | (a << 8) | a, np.uint32)


def test_uniformly_lit_floor_analytic_radiance(orc):
    dim, res = 32, 512
    lum = [4.4, 3.72, 3.24]
    light = orc.make_light(lum, [0.0, -1.0, 0.0])
    for byte in (255, 128):
        tri, alb = _floor_scene(byte)
        f = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), dim, [0.0, -1.0, 0.0])
        sd = orc.shadow_depth(orc.raster(orc.frame_matrix(f), res, res, tri))
        rgba, cnt = orc.voxelize(f, dim, res, tri, alb, light, sd)
        occ = cnt > 0
        assert occ.sum() > 300
        a = (byte / 255.0) ** 2.2
        for ch in range(3):
            assert np.allclose(rgba[..., ch][occ], float(np.float32(lum[ch])) * a, rtol=1e-12)
        assert np.all(rgba[..., 3][occ] == 1.0) and np.all(rgba[~occ] == 0.0)


def test_occluder_shadows_the_floor_analytically(orc):
    dim, res = 32, 512
    tri, alb = _floor_scene(255, occluder=True)
    light = orc.make_light([1, 1, 1], [0.0, -1.0, 0.0])
    f = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), dim, [0.0, -1.0, 0.0])
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(f), res, res, tri))
    rgba, cnt = orc.voxelize(f, dim, res, tri, alb, light, sd)
    vs, org = f.voxel_size, f.origin[0]
    floor_k = {k for k, j, i in zip(*np.nonzero(cnt)) if abs(org + (j + 0.5) * vs) < vs}
    assert floor_k
    xs = org + (np.arange(dim) + 0.5) * vs
    for (k, j, i) in zip(*np.nonzero(cnt)):
        y = org + (j + 0.5) * vs
        if abs(y) > vs:
            continue  # roof voxels
        x = xs[i]
        if x < -vs:  # under the roof
            assert rgba[k, j, i, 0] == 0.0
        elif x > vs:
            assert rgba[k, j, i, 0] == 1.0


def test_voxelize_order_independent(orc):
    import final184_gb300 as g

    sc = g.SyntheticScene(184, 4000, 40)
    f = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), 32, sc.light.direction)
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(f), 256, 256, sc.tri_xyz))
    light = orc.make_light(list(sc.light.luminance), list(sc.light.direction))
    a, ca = orc.voxelize(f, 32, 256, sc.tri_xyz, sc.albedo, light, sd)
    perm = np.random.default_rng(0).permutation(sc.ntris)
    b, cb = orc.voxelize(f, 32, 256, sc.tri_xyz.reshape(-1, 9)[perm].ravel(), sc.albedo[perm], light, sd)
    assert np.array_equal(ca, cb)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-15)


# ---------------- mips and cones ----------------

def test_mip_is_2x2x2_mean(orc):
    rng = np.random.default_rng(4)
    l0 = rng.uniform(0, 1, size=(16, 16, 16, 4))
    _, lv = orc.mip(l0, 5)
    want = l0.reshape(8, 2, 8, 2, 8, 2, 4).mean(axis=(1, 3, 5))
    assert np.allclose(lv[1], want, rtol=1e-14)
    assert np.allclose(lv[4][0, 0, 0], l0.reshape(-1, 4).mean(axis=0))


def test_aniso_mip_composites_front_to_back(orc):
    l0 = np.zeros((4, 4, 4, 4))
    l0[:, :, 0] = [1.0, 0.0, 0.0, 1.0]  # opaque red slab at x = 0
    l0[:, :, 1] = [0.0, 1.0, 0.0, 1.0]  # opaque green slab at x = 1
    _, lv = orc.mip(l0, 2, aniso=True)
    plus_x, minus_x = lv[1][0], lv[1][1]
    assert np.allclose(plus_x[0, 0, 0], [1, 0, 0, 1])  # travelling +x meets red first
    assert np.allclose(minus_x[0, 0, 0], [0, 1, 0, 1])  # travelling -x meets green first
    assert np.allclose(lv[1][2][0, 0, 0], [0.5, 0.5, 0, 1])  # along y both columns average


def test_constant_density_transmittance(orc):
    dim, levels, a, c = 64, 6, 0.05, 0.3
    chain = np.concatenate([np.tile([c, c, c, a], (dim >> l) ** 3) for l in range(levels)])
    p = orc.default_params()
    p.max_distance = 20.0
    p.alpha_stop = 0.9999
    tan_half = 0.1
    o = np.array([32.0, 32.0, 32.0])
    out = orc.cone(chain, dim, levels, o, [1.0, 0.0, 0.0], tan_half, p)
    # the same step schedule in Python: every sample sits wholly inside the grid and reads (c, c, c, a)
    t, n = float(p.start_offset), 0
    while t <= p.max_distance:
        d = max(1.0, 2.0 * t * tan_half)
        n += 1
        t += float(np.float32(p.step_factor)) * d
    assert np.isclose(out[3], 1.0 - (1.0 - a) ** n, rtol=1e-12)
    assert np.isclose(out[0], c * (1.0 - (1.0 - a) ** n) / a, rtol=1e-12)


def test_cone_outside_grid_is_zero(orc):
    dim, levels = 32, 5
    chain = np.concatenate([np.tile([1.0, 1.0, 1.0, 0.5], (dim >> l) ** 3) for l in range(levels)])
    out = orc.cone(chain, dim, levels, [-100.0, 16.0, 16.0], [-1.0, 0.0, 0.0], 0.5)
    assert np.all(out == 0.0)
