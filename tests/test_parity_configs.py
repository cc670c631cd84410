"""The benchmarked configurations against the FP64 oracle (run on a GPU).

- plain-large: the bench's headline request (500k-triangle seeded scene, 2000 objects, 256^3 grid, 8 levels,
  2048^2 shadow map, 1920x1080 view, 5 diffuse + 1 specular cone).  The device voxelizes, builds the chain,
  rasterizes the G-buffer and traces the whole view; the oracle voxelizes the same triangles, builds the chain and
  traces every pixel of the device's G-buffer in FP64.  Occupancy and counts bit-exact; FP32 and FP16 chains within
  REL_TOL as true relative error per value above the near-black floor (oracle/errstats.py).
- served: requests of the served form (FP16 storage, resident weights, rigid moves -> dirty-brick
  re-voxelization + relight + mip rebuild, one trace launch per batch) on resident 128^3 and 256^3 grids; every
  view of every request against the oracle run on that request's own moved geometry.
- batched: one batch over scenes of 64^3, 128^3 and 256^3 grids with views of different sizes (one trace launch),
  each view against the oracle.
"""
import numpy as np
import pytest

from gi_case import clip_matrix, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu

PLAIN_LARGE = dict(seed=1184, ntris=500000, nobjects=2000, dim=256, levels=8, shadow_res=2048, width=1920,
                   height=1080)


def oracle_chain(orc, sc, dim, levels, res, tri=None):
    tri = sc.tri_xyz if tri is None else tri
    b = sc.bounds
    fo = orc.grid_frame(orc.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim,
                        np.array(sc.light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, tri))
    l0, cnt = orc.voxelize(fo, dim, res, tri, sc.albedo,
                           orc.make_light(list(sc.light.luminance), list(sc.light.direction)), sd)
    chain, _ = orc.mip(l0, levels)
    return fo, chain, cnt


class DeviceView:
    """A G-buffer rasterized on the device for one camera, an FP32 output, and host copies for the oracle."""

    def __init__(self, g, gi, torch, tri_d, rough_d, ntris, V, W, H):
        dev = tri_d.device
        n = W * H
        self.W, self.H, self.V = W, H, V
        self.P = g.perspective(59.0, W / H, 0.1, 100.0)
        self.depth = torch.empty(n, dtype=torch.float32, device=dev)
        self.normal = torch.empty(n, dtype=torch.int32, device=dev)
        self.rough = torch.empty(n, dtype=torch.int16, device=dev)
        self.out = torch.zeros(2 * n * 4, dtype=torch.float32, device=dev)
        self.view = g.make_view(V, self.P, W, H, self.depth.data_ptr(), self.normal.data_ptr(), self.rough.data_ptr(),
                                self.out.data_ptr())
        gi.gbuffer(tri_d.data_ptr(), rough_d.data_ptr(), ntris, self.view)

    def host(self):
        H, W = self.H, self.W
        return (self.depth.cpu().numpy().reshape(H, W), self.normal.cpu().numpy().view(np.uint32).reshape(H, W),
                self.rough.cpu().numpy().view(np.uint16).reshape(H, W))

    def result(self):
        return self.out.cpu().numpy().reshape(2, self.H, self.W, 4)

    def oracle(self, orc, fo, dim, levels, chain):
        dep, nrm, rgh = self.host()
        return orc.trace(fo, dim, levels, chain, self.V, self.P, self.W, self.H, dep, nrm, rgh)


def test_plain_large_fp32_and_fp16_vs_fp64(lib, orc):
    import torch

    import final184_gb300 as g

    cfg = PLAIN_LARGE
    dev = torch.device("cuda", 0)
    sc = g.SyntheticScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    dim, levels, res, W, H = cfg["dim"], cfg["levels"], cfg["shadow_res"], cfg["width"], cfg["height"]
    gi = g.VoxelGI(0)
    tri = torch.from_numpy(sc.tri_xyz).to(dev)
    alb = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    rough = torch.from_numpy(sc.roughness).to(dev)
    v = DeviceView(g, gi, torch, tri, rough, sc.ntris, g.look_at(sc.eye, sc.target), W, H)
    got, counts = {}, None
    for fmt in (g.FMT_F32, g.FMT_F16):
        grid = gi.create_grid(dim, levels, fmt, 0, res, g.GRID_KEEP_COUNTS if fmt == g.FMT_F32 else 0)
        gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
        gi.mip(grid)
        gi.trace(grid, [v.view])
        gi.sync()
        got[fmt] = v.result().copy()
        if fmt == g.FMT_F32:
            counts = gi.read_counts(grid)
        gi.destroy_grid(grid)
    fo, chain, cnt = oracle_chain(orc, sc, dim, levels, res)
    assert np.array_equal(counts, cnt), "occupancy / counts differ in %d voxels" % int((counts != cnt).sum())
    ref = v.oracle(orc, fo, dim, levels, chain)
    gi.close()
    assert ref[0, ..., :3].mean() > 1e-3  # lit
    for fmt, name in ((g.FMT_F32, "fp32"), (g.FMT_F16, "fp16")):
        e = rel_err(got[fmt], ref)
        print("plain-large %s chain, %dx%d vs FP64:" % (name, W, H), e)
        assert e.ok(), "%s: %s" % (name, e)


SERVED_SCENES = [(128, 7, 100000, 400, 4242), (256, 8, 300000, 1200, 4442)]  # dim, levels, tris, objects, seed


def served_moves(rng, sc, fraction=0.05):
    n = int(rng.integers(1, int(fraction * (sc.nobjects - 1)) + 1))
    moves = []
    for o in rng.choice(np.arange(1, sc.nobjects), n, replace=False):
        moves.append((int(sc.object_first[o]), int(sc.object_count[o]),
                      [float(x) for x in rng.uniform(-0.2, 0.2, 3).astype(np.float32)]))
    return moves


def apply_moves(tri, moves):
    """The caller-side copy of the moves: the same FP32 additions the device applies."""
    for f, c, off in moves:
        seg = tri[f * 9:(f + c) * 9].reshape(-1, 3)
        seg += np.asarray(off, dtype=np.float32)


def test_served_requests_vs_fp64(lib, orc):
    """Two requests per scene, each moving objects (dirty bricks re-voxelized, grid relit, mips rebuilt), the
    second one after the first's moves: every view against the oracle on that request's geometry."""
    import torch

    import final184_gb300 as g

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(77)
    srv = g.Server(0, slots=2, max_batch_views=16)
    gi = g.VoxelGI(0)
    scenes = []
    for k, (dim, levels, ntris, nobj, seed) in enumerate(SERVED_SCENES):
        sc = g.SyntheticScene(seed, ntris, nobj)
        srv.add_scene(k, g.GridDesc(dim, levels, g.FMT_F16, 0, 2048, 0), sc.tri_xyz, sc.albedo, sc.bounds, sc.light)
        scenes.append((sc, dim, levels, sc.tri_xyz.copy()))
    checked = 0
    for step in range(2):
        for k, (sc, dim, levels, geo) in enumerate(scenes):
            moves = served_moves(rng, sc)
            apply_moves(geo, moves)
            tri = torch.from_numpy(geo).to(dev)
            rough = torch.from_numpy(sc.roughness).to(dev)
            views = []
            for j, (W, H) in enumerate([(512, 288), (384, 384)]):
                eye, tgt = sc.camera(10 * step + j)
                views.append(DeviceView(g, gi, torch, tri, rough, sc.ntris, g.look_at(eye, tgt), W, H))
            gi.sync()
            r = srv.wait(srv.submit(k, [v.view for v in views], moves))
            assert r.status == 0
            torch.cuda.synchronize()
            fo, chain, _ = oracle_chain(orc, sc, dim, levels, 2048, tri=geo)
            for v in views:
                ref = v.oracle(orc, fo, dim, levels, chain)
                e = rel_err(v.result(), ref)
                print("served %d^3 request %d (%d objects moved), %dx%d:" % (dim, step, len(moves), v.W, v.H), e)
                assert e.ok(), str(e)
                checked += 1
    srv.close()
    gi.close()
    assert checked == 8


BATCH_SCENES = [(64, 6, 20000, 80, 3184), (128, 7, 150000, 600, 3201), (256, 8, 400000, 1600, 3218)]


def test_batched_slice_vs_fp64(lib, orc):
    """Three resident scenes (64^3, 128^3, 256^3) with 1-3 views of mixed sizes, all traced in one launch."""
    import torch

    import final184_gb300 as g

    dev = torch.device("cuda", 0)
    srv = g.Server(0, slots=1, max_batch_views=64)
    gi = g.VoxelGI(0)
    reqs, keep = [], []
    sizes = [[(256, 256)], [(640, 360), (300, 500)], [(1024, 576), (256, 320), (480, 270)]]
    for k, (dim, levels, ntris, nobj, seed) in enumerate(BATCH_SCENES):
        sc = g.SyntheticScene(seed, ntris, nobj)
        srv.add_scene(k, g.GridDesc(dim, levels, g.FMT_F16, 0, min(2048, dim * 16), 0), sc.tri_xyz, sc.albedo,
                      sc.bounds, sc.light)
        tri = torch.from_numpy(sc.tri_xyz).to(dev)
        rough = torch.from_numpy(sc.roughness).to(dev)
        views = []
        for j, (W, H) in enumerate(sizes[k]):
            eye, tgt = sc.camera(j)
            views.append(DeviceView(g, gi, torch, tri, rough, sc.ntris, g.look_at(eye, tgt), W, H))
        keep.append((sc, dim, levels, views))
        reqs.append((k, [v.view for v in views], []))
    gi.sync()
    res = [srv.wait(t) for t in srv.submit_many(reqs)]
    assert all(r.status == 0 for r in res)
    assert len({r.batch for r in res}) == 1  # one batch, one trace launch
    torch.cuda.synchronize()
    for sc, dim, levels, views in keep:
        fo, chain, _ = oracle_chain(orc, sc, dim, levels, min(2048, dim * 16))
        for v in views:
            e = rel_err(v.result(), v.oracle(orc, fo, dim, levels, chain))
            print("batched %d^3 %dx%d:" % (dim, v.W, v.H), e)
            assert e.ok(), str(e)
    srv.close()
    gi.close()
