"""CUDA path vs the CPU oracle on seeded scenes (run on a GPU).

Bit-exact: grid frame, shadow map, voxel occupancy and contribution counts, G-buffer depth and triangle ids,
grid bytes under a shuffled triangle order, dirty-brick re-voxelization vs full voxelization.
Within REL_TOL (1e-3 true relative error per value above the near-black floor, oracle/errstats.py): injected
radiance, mip levels, cone-traced pixels.
"""
import numpy as np
import pytest

from gi_case import REL_TOL, Case, clip_matrix, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(lib):
    c = Case()
    c.voxelize()
    c.mip()
    c.gbuffer()
    return c


@pytest.fixture(scope="module")
def oracle_l0(case, orc):
    fo = case.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), case.res, case.res, case.sc.tri_xyz))
    l0, cnt = orc.voxelize(fo, case.dim, case.res, case.sc.tri_xyz, case.sc.albedo, case.oracle_light(), sd)
    return fo, sd, l0, cnt


def test_frame_host_device_oracle_identical(case, oracle_l0):
    fo = oracle_l0[0]
    fd = case.gi.frame(case.grid)
    fh = case.g.frame_from_bounds(case.sc.bounds, case.dim, np.array(case.sc.light.direction, np.float32))
    assert bytes(fd) == bytes(fo)
    assert bytes(fh) == bytes(fo)


def test_frame_from_device_bounds(lib):
    """bounds=None: the AABB is reduced on the device and the frame computed there (given bounds, the host computes
    it); the scene AABB is the room, so the frame is the same, and so is the traced image (the trace reads the
    frame's FP32 pairs, written by the device kernel here and by the host with given bounds)."""
    c = Case(ntris=5000, nobj=40, dim=32, levels=5, res=256, width=64, height=32)
    c.gbuffer()
    c.voxelize(bounds=False)
    fo = c.oracle_frame()
    assert bytes(c.gi.frame(c.grid)) == bytes(fo)
    c.mip()
    img_device_frame = c.trace().copy()
    c.voxelize(bounds=True)
    assert bytes(c.gi.frame(c.grid)) == bytes(fo)
    c.mip()
    img_host_frame = c.trace()
    assert float(np.abs(img_host_frame).sum()) > 0
    assert np.array_equal(img_device_frame.view(np.uint32), img_host_frame.view(np.uint32))


def test_shadow_map_bit_exact(case, oracle_l0):
    sd = oracle_l0[1]
    got = case.gi.read_shadow(case.grid)
    assert got.shape == sd.shape
    assert np.array_equal(got.view(np.uint32), sd.view(np.uint32))
    assert (sd < 1.0).mean() > 0.3  # the map is not trivially empty


def test_voxel_occupancy_and_counts_bit_exact(case, oracle_l0):
    cnt = oracle_l0[3]
    got = case.gi.read_counts(case.grid)
    assert np.array_equal(got > 0, cnt > 0), "occupancy differs in %d voxels" % int(((got > 0) != (cnt > 0)).sum())
    assert np.array_equal(got, cnt)
    l0 = case.gi.read_level(case.grid, 0)
    assert np.array_equal(l0[..., 3] > 0, cnt > 0)


def test_injected_radiance(case, oracle_l0):
    l0_ref = oracle_l0[2]
    l0 = case.gi.read_level(case.grid, 0)
    e = rel_err(l0, l0_ref)
    print("L0 radiance:", e)
    assert e.ok(), str(e)
    lit = (l0_ref[..., 0] > 0).sum()
    assert lit > 1000
    # the scene exercises the carry of the 33.31 fixed-point sums past 32 bits: a lit voxel's sum is
    # count * mean weight * 2^31 with mean weight = radiance / luminance
    lum = np.array(case.oracle_light().luminance[:3], np.float64)
    sums = oracle_l0[3][..., None] * l0_ref[..., :3] / lum * 2.0 ** 31
    assert (sums >= 2.0 ** 32).sum() > 100


def test_mip_chain(case, orc):
    l0 = case.gi.read_level(case.grid, 0).astype(np.float64)
    _, levels = orc.mip(l0, case.levels)
    for lv in range(1, case.levels):
        got = case.gi.read_level(case.grid, lv)
        e = rel_err(got, levels[lv])
        assert e.ok(1e-5), "level %d: %s" % (lv, e)


def test_gbuffer_bit_exact(case, orc):
    keys = orc.raster(clip_matrix(case.P, case.V), case.W, case.H, case.sc.tri_xyz)
    dep, nrm, rgh, tid = orc.gbuffer_resolve(keys, case.sc.tri_xyz, case.sc.roughness, case.V)
    gd, gn, gr, gt = case.gbuffer_host()
    assert np.array_equal(gt, tid)
    assert np.array_equal(gd.view(np.uint32), dep.view(np.uint32))
    assert np.array_equal(gr, rgh)
    # normals: FP32 on the device vs FP64 in the oracle, then rounded to FP16 -> at most one FP16 ulp apart
    dx = np.abs(gn.astype(np.int64) & 0xffff - (nrm.astype(np.int64) & 0xffff))
    assert int(np.abs((gn & 0xffff).astype(np.int64) - (nrm & 0xffff).astype(np.int64)).max()) <= 1
    assert int(np.abs((gn >> 16).astype(np.int64) - (nrm >> 16).astype(np.int64)).max()) <= 1
    del dx


def test_trace_matches_oracle(case, orc, oracle_l0):
    fo = oracle_l0[0]
    got = case.trace()
    dep, nrm, rgh, _ = case.gbuffer_host()
    chain, _ = orc.mip(oracle_l0[2], case.levels)
    ref = orc.trace(fo, case.dim, case.levels, chain, case.V, case.P, case.W, case.H, dep, nrm, rgh)
    e = rel_err(got, ref)
    print("trace:", e)
    assert e.ok(), str(e)
    assert ref[0, ..., :3].mean() > 1e-3  # lit scene


def test_trace_count_outputs_and_totals(case, orc, oracle_l0):
    """The instrumented trace writes the plain trace's bytes, and its step / level-sample totals equal the FP32
    oracle's over the same chain (read back from the device) up to a few cones whose exit test sits within an ulp
    of the grid margin."""
    ref_img = case.trace().copy()
    steps, samples = case.gi.trace_count(case.grid, [case.view])
    case.gi.sync()
    got = case.out.cpu().numpy().reshape(2, case.H, case.W, 4)
    assert np.array_equal(got.view(np.uint32), ref_img.view(np.uint32))
    chain = np.concatenate([case.gi.read_level(case.grid, l).ravel() for l in range(case.levels)])
    dep, nrm, rgh, _ = case.gbuffer_host()
    _, osteps, osamples = orc.trace_count(oracle_l0[0], case.dim, case.levels, chain, case.V, case.P, case.W, case.H,
                                          dep, nrm, rgh)
    lit = int((dep < 1.0).sum())
    print("steps/px %.2f (oracle %.2f), samples/px %.2f (oracle %.2f)" % (steps / lit, osteps / lit, samples / lit,
                                                                          osamples / lit))
    assert 10 * lit < steps < 400 * lit and steps <= samples <= 2 * steps
    assert abs(steps - osteps) <= 1e-4 * osteps and abs(samples - osamples) <= 1e-4 * osamples


def test_shuffled_triangle_order_bit_identical(case):
    rng = np.random.default_rng(7)
    perm = rng.permutation(case.sc.ntris)
    base = case.gi.read_level(case.grid, 0).copy()
    c2 = Case(keep_counts=False)
    tri = case.sc.tri_xyz.reshape(-1, 9)[perm].ravel()
    alb = case.sc.albedo[perm]
    c2.upload(tri, alb)
    c2.voxelize()
    got = c2.gi.read_level(c2.grid, 0)
    assert np.array_equal(got.view(np.uint32), base.view(np.uint32))


def test_dirty_brick_revoxelize_equals_full(lib):
    c = Case(ntris=20000, nobj=200, dim=64, levels=6, res=1024, keep_counts=False)
    c.voxelize()
    moved = c.sc.move_objects(99, 0.05, 1.0)
    assert len(moved) > 0
    # dirty bricks: every brick (a superset is always correct); then a real subset
    nb = (c.dim // 8) ** 3
    c.upload(c.sc.tri_xyz, c.sc.albedo)
    c.voxelize(dirty=np.arange(nb, dtype=np.uint32))
    inc = c.gi.read_level(c.grid, 0).copy()
    full = Case(ntris=20000, nobj=200, dim=64, levels=6, res=1024, keep_counts=False)
    full.sc.move_objects(99, 0.05, 1.0)
    full.upload(full.sc.tri_xyz, full.sc.albedo)
    full.voxelize()
    ref = full.gi.read_level(full.grid, 0)
    assert np.array_equal(inc.view(np.uint32), ref.view(np.uint32))


def _chain_bytes(c):
    return [c.gi.read_level(c.grid, lv).view(np.uint32).copy() for lv in range(c.levels)]


@pytest.mark.parametrize("dim,levels", [(64, 6), (16, 4), (32, 2)])
def test_mip_from_voxelized_low_levels_equals_build_from_l0(lib, dim, levels):
    """Isotropic FP32 grids: the voxelization writes each brick's block of levels 1..3 with L0 and the mip goes on
    from level 3.  The chain equals a build from L0 (forced by handing out a level pointer), after a full
    voxelization and after dirty-brick updates (all bricks, and an arbitrary half of them)."""
    c = Case(ntris=20000, nobj=200, dim=dim, levels=levels, res=1024, keep_counts=False)
    nb = (dim // 8) ** 3
    for dirty in (None, np.arange(nb, dtype=np.uint32), np.arange(0, nb, 2, dtype=np.uint32)):
        if dirty is not None:
            c.sc.move_objects(7 + len(dirty), 0.05, 1.0)
            c.upload(c.sc.tri_xyz, c.sc.albedo)
        c.voxelize(dirty=dirty)
        c.mip()
        continued = _chain_bytes(c)
        assert np.abs(c.gi.read_level(c.grid, min(1, levels - 1))).sum() > 0
        c.gi.level_ptr(c.grid, 0)
        c.mip()
        rebuilt = _chain_bytes(c)
        for lv in range(levels):
            assert np.array_equal(continued[lv], rebuilt[lv]), "level %d differs (dirty=%s)" % (
                lv, None if dirty is None else len(dirty))


def test_partial_mip_after_voxelized_low_levels(lib):
    """f184gi_mip with fewer levels than the grid after a voxelization that wrote levels 1..3: the levels asked for
    equal a build from L0, whether they end inside the voxelized ones (2) or beyond them (5)."""
    c = Case(ntris=20000, nobj=200, dim=64, levels=6, res=1024, keep_counts=False)
    c.voxelize()
    c.mip()
    full = _chain_bytes(c)
    for n in (2, 5):
        c.voxelize()
        c.gi.mip(c.grid, levels=n)
        c.gi.sync()
        for lv in range(n):
            assert np.array_equal(c.gi.read_level(c.grid, lv).view(np.uint32), full[lv]), (n, lv)


def test_fp16_storage_trace_error(lib, orc):
    c = Case(fmt=1)
    c.voxelize()
    c.mip()
    c.gbuffer()
    got = c.trace()
    fo = c.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), c.res, c.res, c.sc.tri_xyz))
    l0, _ = orc.voxelize(fo, c.dim, c.res, c.sc.tri_xyz, c.sc.albedo, c.oracle_light(), sd)
    chain, _ = orc.mip(l0, c.levels)
    dep, nrm, rgh, _ = c.gbuffer_host()
    ref = orc.trace(fo, c.dim, c.levels, chain, c.V, c.P, c.W, c.H, dep, nrm, rgh)
    e = rel_err(got, ref)
    print("fp16 storage trace:", e)
    assert e.ok(), str(e)


@pytest.mark.parametrize("fmt", [0, 1], ids=["fp32", "fp16"])
def test_anisotropic_chain_and_trace(lib, orc, fmt):
    """Six-direction mips (level 0 -> 6 volumes per level) and the anisotropic cone trace against the oracle."""
    c = Case(fmt=fmt, aniso=True)
    c.voxelize()
    c.mip()
    c.gbuffer()
    l0 = c.gi.read_level(c.grid, 0).astype(np.float64)
    _, levels = orc.mip(l0, c.levels, aniso=True)
    for lv in range(1, c.levels):
        for d in range(6):
            got = c.gi.read_level(c.grid, lv, direction=d)
            if fmt == 0:
                e = rel_err(got, levels[lv][d])
                assert e.ok(1e-5), "level %d direction %d: %s" % (lv, d, e)
                continue
            # FP16 storage: binary16 radiance rounds at every level (2^-11 relative each; the composite
            # f + (1 - f.a) b adds one more), unorm16 opacity by half a step (2^-17 absolute) each
            e = rel_err(got[..., :3], levels[lv][d][..., :3])
            assert e.ok((lv + 1) * 2.0 ** -11), "level %d direction %d radiance: %s" % (lv, d, e)
            da = np.abs(got[..., 3].astype(np.float64) - levels[lv][d][..., 3]).max()
            assert da <= (lv + 1) * 2.0 ** -17, "level %d direction %d opacity: %.3g" % (lv, d, da)
    got = c.trace()
    fo = c.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), c.res, c.res, c.sc.tri_xyz))
    ol0, _ = orc.voxelize(fo, c.dim, c.res, c.sc.tri_xyz, c.sc.albedo, c.oracle_light(), sd)
    chain, _ = orc.mip(ol0, c.levels, aniso=True)
    dep, nrm, rgh, _ = c.gbuffer_host()
    ref = orc.trace(fo, c.dim, c.levels, chain, c.V, c.P, c.W, c.H, dep, nrm, rgh, aniso=True)
    e = rel_err(got, ref)
    print("anisotropic %s trace:" % ["fp32", "fp16"][fmt], e)
    assert e.ok(), str(e)
    assert ref[0, ..., :3].mean() > 1e-3  # lit scene


@pytest.mark.parametrize("seed,ntris,nobj,dim,res", [(11, 20000, 20, 64, 512), (12, 30000, 8, 128, 1024),
                                                     (14, 8000, 3, 64, 512), (16, 20000, 50, 32, 256)])
def test_counts_and_shadow_bit_exact_across_scenes(lib, orc, seed, ntris, nobj, dim, res):
    """Scenes of few large objects (long triangles crossing many bricks: the voxelizer's 64-bit edge tests and its
    items spread over several threads) and of many small ones: occupancy/counts and the shadow map bit-exact."""
    import torch

    import final184_gb300 as g

    dev = torch.device("cuda:0")
    gi = g.VoxelGI(0)
    sc = g.SyntheticScene(seed, ntris, nobj)
    tri = torch.from_numpy(sc.tri_xyz).to(dev)
    alb = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    grid = gi.create_grid(dim, 5, g.FMT_F32, 0, res, g.GRID_KEEP_COUNTS)
    gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
    gi.sync()
    cnt, shadow = gi.read_counts(grid), gi.read_shadow(grid)
    gi.close()
    b = sc.bounds
    fo = orc.grid_frame(orc.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim,
                        np.array(sc.light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, sc.tri_xyz))
    _, ocnt = orc.voxelize(fo, dim, res, sc.tri_xyz, sc.albedo,
                           orc.make_light(list(sc.light.luminance), list(sc.light.direction)), sd)
    assert int((ocnt > 0).sum()) > 1000
    assert np.array_equal(cnt, ocnt), "counts differ in %d voxels" % int((cnt != ocnt).sum())
    assert np.array_equal(shadow.view(np.uint32), sd.astype(np.float32).view(np.uint32))
