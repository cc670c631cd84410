"""The precision form on a GPU against the FP64 oracle: 2M-triangle seeded scene, 512^3 FP16 chain in 8^3 Morton
bricks with six-direction anisotropic mips (9 levels), 4096^2 shadow map, 3840x2160 G-buffer.

The oracle voxelizes the whole scene and builds the anisotropic chain in FP64, then traces every 64th row of the
device's own G-buffer; the device output must be within REL_TOL (true relative error per value above the
near-black floor, oracle/errstats.py) of it.  This is the error that the precision leg of bench.py runs under.
"""
import numpy as np
import pytest

from gi_case import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

PRECISION = dict(seed=2184, ntris=2000000, nobjects=8000, dim=512, levels=9, shadow_res=4096, width=3840,
                 height=2160)


def test_precision_form_error_vs_fp64(lib, orc):
    import torch

    import final184_gb300 as g

    cfg = PRECISION
    dev = torch.device("cuda", 0)
    sc = g.SyntheticScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    gi = g.VoxelGI(0)
    grid = gi.create_grid(cfg["dim"], cfg["levels"], g.FMT_F16, 1, cfg["shadow_res"])
    tri = torch.from_numpy(sc.tri_xyz).to(dev)
    alb = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    rough = torch.from_numpy(sc.roughness).to(dev)
    W, H, dim, levels, res = cfg["width"], cfg["height"], cfg["dim"], cfg["levels"], cfg["shadow_res"]
    n = W * H
    V, P = g.look_at(sc.eye, sc.target), g.perspective(59.0, W / H, 0.1, 100.0)
    depth = torch.empty(n, dtype=torch.float32, device=dev)
    normal = torch.empty(n, dtype=torch.int32, device=dev)
    rgh = torch.empty(n, dtype=torch.int16, device=dev)
    out = torch.empty(2 * n * 4, dtype=torch.float32, device=dev)
    view = g.make_view(V, P, W, H, depth.data_ptr(), normal.data_ptr(), rgh.data_ptr(), out.data_ptr())
    gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view)
    gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
    gi.mip(grid)
    gi.trace(grid, [view])
    gi.sync()
    got = out.cpu().numpy().reshape(2, H, W, 4)
    dep = depth.cpu().numpy().reshape(H, W)
    nrm = normal.cpu().numpy().view(np.uint32).reshape(H, W)
    rg = rgh.cpu().numpy().view(np.uint16).reshape(H, W)
    gi.close()

    b = sc.bounds
    fo = orc.grid_frame(orc.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim,
                        np.array(sc.light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, sc.tri_xyz))
    l0, _ = orc.voxelize(fo, dim, res, sc.tri_xyz, sc.albedo,
                         orc.make_light(list(sc.light.luminance), list(sc.light.direction)), sd)
    chain, _ = orc.mip(l0, levels, aniso=True)
    del l0
    rows = list(range(0, H, 64))
    ref = np.stack([orc.trace(fo, dim, levels, chain, V, P, W, H, dep, nrm, rg, rows=(r, r + 1), aniso=True)[:, r]
                    for r in rows], axis=1)
    e = rel_err(got[:, rows], ref)
    print("precision form vs FP64: %d rows," % len(rows), e)
    assert e.ok(), str(e)
    assert ref[0, ..., :3].mean() > 1e-4  # lit
