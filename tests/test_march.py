"""The reference-faithful mode: the reference's 565 voxel volume and its single-ray march.

CPU: known answers for the volume (dominant-axis raster, VoxelPS swizzles and packing, last triangle wins), the
sample-angle sin/cos, and the FP32 restatement against the FP64 one.  GPU: the volume and the marched image are
bit-identical to the oracle's FP32 restatement (the device's operation sequence).
"""
import numpy as np
import pytest


def _frame(orc, dim, lo=-10.0, hi=10.0, light=(0.3, -1.0, 0.2)):
    return orc.grid_frame(orc.make_bounds((lo, lo, lo), (hi, hi, hi)), dim, np.array(light, np.float32))


def _quad(y, x0=-10.0, x1=10.0, z0=-10.0, z1=10.0):
    """Two triangles of the horizontal square at height y."""
    return np.array([[x0, y, z0, x1, y, z0, x1, y, z1], [x0, y, z0, x1, y, z1, x0, y, z1]], np.float32)


def test_sample_angle_sincos(orc):
    v = np.linspace(0.0, 1.0, 20001, endpoint=False, dtype=np.float32)
    got = np.array([orc.sincos_turns(x) for x in v])
    ref = np.stack([np.sin(2 * np.pi * v.astype(np.float64)), np.cos(2 * np.pi * v.astype(np.float64))], 1)
    assert np.abs(got - ref).max() < 2e-7


def test_floor_quad_voxels_and_packing(orc):
    dim = 32
    fr = _frame(orc, dim)
    tri = _quad(0.0)
    alb = np.array([0x00FF8040, 0x00FF8040], np.uint32)  # r = 0x40, g = 0x80, b = 0xFF
    vol = orc.refvox(fr, dim, tri, alb)
    occ = np.argwhere(vol != 0)  # (z, y, x)
    # a floor is Y-dominant: every pixel (x, z) of the grid's footprint lands in one y layer
    assert len(np.unique(occ[:, 1])) == 1
    u_y = (0.0 - fr.origin[1]) / fr.voxel_size  # the quad's voxel coordinate
    assert occ[0, 1] == int(np.float32(u_y / dim) * np.float32(dim - 1))
    color = (int(np.float32(0x40 / 255.0) * np.float32(31)) << 11) | (int(np.float32(0x80 / 255.0) * np.float32(63)) << 5) \
        | int(np.float32(1.0) * np.float32(31))
    nrm = [int(vol[tuple(o)]) >> 16 for o in occ]
    assert all((int(vol[tuple(o)]) & 0xFFFF) == color for o in occ)
    # face normal (0, +-1, 0): x and z fields 15, y field 63 (up) or 0 (down, clamped at 0)
    assert set(nrm) <= {(15 << 11) | (63 << 5) | 15, (15 << 11) | (0 << 5) | 15}


def test_last_triangle_wins(orc):
    dim = 32
    fr = _frame(orc, dim)
    tri = np.concatenate([_quad(0.0), _quad(0.0)])
    alb = np.array([0x000000FF] * 2 + [0x0000FF00] * 2, np.uint32)
    vol = orc.refvox(fr, dim, tri, alb)
    occ = vol[vol != 0] & 0xFFFF
    assert len(occ) > 0 and np.all(occ == (63 << 5))  # green: the second quad's colour


def test_march_fp32_restatement_matches_fp64(orc, lib):
    import final184_gb300 as g
    from gi_case import clip_matrix

    sc = g.SyntheticScene(184, 20000, 200)
    dim, res, W, H = 64, 512, 96, 64
    b = sc.bounds
    fr = orc.grid_frame(orc.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim,
                        np.array(sc.light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fr), res, res, sc.tri_xyz))
    vol = orc.refvox(fr, dim, sc.tri_xyz, sc.albedo)
    V, P = g.look_at(sc.eye, sc.target), g.perspective(59.0, W / H, 0.1, 100.0)
    keys = orc.raster(clip_matrix(P, V), W, H, sc.tri_xyz)
    dep, nrm, _, _ = orc.gbuffer_resolve(keys, sc.tri_xyz, sc.roughness, V)
    light = orc.make_light(list(sc.light.luminance), list(sc.light.direction))
    a = orc.march(fr, dim, vol, sd, light, V, P, W, H, dep, nrm)
    b64 = orc.march(fr, dim, vol, sd, light, V, P, W, H, dep, nrm, f64=True)
    e = np.abs(a[..., :3] - b64[..., :3]) / np.maximum(np.abs(b64[..., :3]), 1e-2)
    # discrete events (a step that lands in the next voxel in one precision only) change a few pixels
    assert (e < 1e-3).mean() > 0.97
    assert float(b64[..., :3].mean()) > 1e-3


@pytest.mark.gpu
def test_gpu_volume_and_march_bit_identical_to_the_restatement(lib, orc):
    import torch

    import final184_gb300 as g
    from gi_case import Case

    c = Case()
    dim = 128
    grid = c.gi.create_grid(dim, 1, g.FMT_RG16, 0, c.res)
    c.gi.voxelize(grid, c.tri_d.data_ptr(), c.alb_d.data_ptr(), c.ntris, c.sc.light, bounds=c.sc.bounds)
    c.gbuffer()
    out = torch.zeros(c.W * c.H * 4, dtype=torch.float32, device=c.dev)
    view = g.make_view(c.V, c.P, c.W, c.H, c.depth.data_ptr(), c.normal.data_ptr(), c.rgh.data_ptr(),
                       out.data_ptr())
    c.gi.march(grid, [view])
    c.gi.sync()
    vol = c.gi.read_level(grid, 0)
    fr = orc.grid_frame(orc.make_bounds((c.sc.bounds.min.x, c.sc.bounds.min.y, c.sc.bounds.min.z),
                                        (c.sc.bounds.max.x, c.sc.bounds.max.y, c.sc.bounds.max.z)), dim,
                        np.array(c.sc.light.direction, np.float32))
    ref_vol = orc.refvox(fr, dim, c.sc.tri_xyz, c.sc.albedo)
    assert np.array_equal(vol, ref_vol)
    assert (vol != 0).mean() > 0.01
    sd = c.gi.read_shadow(grid)
    dep, nrm, _, _ = c.gbuffer_host()
    light = orc.make_light(list(c.sc.light.luminance), list(c.sc.light.direction))
    ref = orc.march(fr, dim, ref_vol, sd, light, c.V, c.P, c.W, c.H, dep, nrm)
    got = out.cpu().numpy().reshape(c.H, c.W, 4)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    ref64 = orc.march(fr, dim, ref_vol, sd, light, c.V, c.P, c.W, c.H, dep, nrm, f64=True)
    e = np.abs(got[..., :3] - ref64[..., :3]) / np.maximum(np.abs(ref64[..., :3]), 1e-2)
    print("march vs FP64: %.4f of values within 1e-3, max %.3g" % ((e < 1e-3).mean(), e.max()))
    # another frame seed draws other rays
    p = g.default_march_params()
    p.frame = 7
    c.gi.march(grid, [view], params=p)
    c.gi.sync()
    assert not np.array_equal(out.cpu().numpy().reshape(c.H, c.W, 4), got)
