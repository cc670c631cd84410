"""Golden fixture (tests/golden/small_scene.npz, made by tests/golden/make_golden.py from the FP64 oracle).

CPU: the oracle reproduces the fixture from the fixture's own inputs (regression pin of the oracle).
GPU: the CUDA path, fed the fixture's inputs through the C ABI, matches the fixture: shadow map, counts and the
G-buffer exactly, injected radiance and traced pixels within REL_TOL.
"""
import os

import numpy as np
import pytest

from gi_case import REL_TOL, clip_matrix, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "small_scene.npz")))


def test_oracle_reproduces_golden(orc, gold):
    dim, levels, res, W, H = (int(x) for x in gold["dims"])
    fo = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), dim, gold["ldir"])
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, gold["tri"]))
    assert np.array_equal(sd.view(np.uint32), gold["shadow"].view(np.uint32))
    l0, cnt = orc.voxelize(fo, dim, res, gold["tri"], gold["albedo"], orc.make_light(gold["lum"], gold["ldir"]), sd)
    assert np.array_equal(cnt, gold["counts"])
    assert np.allclose(l0, gold["l0"], rtol=1e-12, atol=0)
    chain, _ = orc.mip(l0, levels)
    gk = orc.raster(clip_matrix(gold["proj"], gold["view"]), W, H, gold["tri"])
    dep, nrm, rgh, tid = orc.gbuffer_resolve(gk, gold["tri"], gold["rough"], gold["view"])
    assert np.array_equal(tid, gold["tri_id"]) and np.array_equal(dep.view(np.uint32), gold["depth"].view(np.uint32))
    out = orc.trace(fo, dim, levels, chain, gold["view"], gold["proj"], W, H, gold["depth"], gold["normal"],
                    gold["rough_px"])
    assert np.allclose(out, gold["trace"], rtol=1e-12, atol=1e-15)


def test_oracle_trace_count_same_image(orc, gold):
    """The counting oracle trace returns the plain FP32 trace's image and positive, consistent totals."""
    dim, levels, res, W, H = (int(x) for x in gold["dims"])
    fo = orc.grid_frame(orc.make_bounds((-10, -10, -10), (10, 10, 10)), dim, gold["ldir"])
    chain, _ = orc.mip(gold["l0"], levels, f64=False)
    args = (fo, dim, levels, chain, gold["view"], gold["proj"], W, H, gold["depth"], gold["normal"], gold["rough_px"])
    plain = orc.trace(*args, f64=False)
    img, steps, samples = orc.trace_count(*args)
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    lit = int((gold["depth"] < 1.0).sum())
    assert 10 * lit < steps < 400 * lit and steps <= samples <= 2 * steps


@pytest.mark.gpu
def test_gpu_matches_golden(lib, gold):
    import torch

    import final184_gb300 as g

    dim, levels, res, W, H = (int(x) for x in gold["dims"])
    dev = torch.device("cuda:0")
    gi = g.VoxelGI(0)
    grid = gi.create_grid(dim, levels, g.FMT_F32, 0, res, g.GRID_KEEP_COUNTS)
    tri = torch.from_numpy(gold["tri"]).to(dev)
    alb = torch.from_numpy(gold["albedo"].view(np.int32)).to(dev)
    rough = torch.from_numpy(gold["rough"]).to(dev)
    light = g.make_light(gold["lum"], gold["ldir"])
    gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), tri.numel() // 9, light,
                bounds=g.make_bounds((-10, -10, -10), (10, 10, 10)))
    gi.mip(grid)
    gi.sync()
    assert np.array_equal(gi.read_shadow(grid).view(np.uint32), gold["shadow"].view(np.uint32))
    assert np.array_equal(gi.read_counts(grid), gold["counts"].astype(np.uint32))
    e = rel_err(gi.read_level(grid, 0), gold["l0"])
    assert e.ok(), str(e)
    # G-buffer raster on the device vs the fixture
    n = W * H
    depth = torch.empty(n, dtype=torch.float32, device=dev)
    normal = torch.empty(n, dtype=torch.int32, device=dev)
    rgh = torch.empty(n, dtype=torch.int16, device=dev)
    tid = torch.empty(n, dtype=torch.int32, device=dev)
    out = torch.empty(2 * n * 4, dtype=torch.float32, device=dev)
    view = g.make_view(gold["view"], gold["proj"], W, H, depth.data_ptr(), normal.data_ptr(), rgh.data_ptr(),
                       out.data_ptr())
    gi.gbuffer(tri.data_ptr(), rough.data_ptr(), tri.numel() // 9, view, tid.data_ptr())
    gi.sync()
    assert np.array_equal(tid.cpu().numpy().view(np.uint32).reshape(H, W), gold["tri_id"])
    assert np.array_equal(depth.cpu().numpy().reshape(H, W).view(np.uint32), gold["depth"].view(np.uint32))
    # trace over the fixture's own G-buffer
    depth.copy_(torch.from_numpy(gold["depth"].ravel()))
    normal.copy_(torch.from_numpy(gold["normal"].ravel().view(np.int32)))
    rgh.copy_(torch.from_numpy(gold["rough_px"].ravel().view(np.int16)))
    gi.trace(grid, [view])
    gi.sync()
    got = out.cpu().numpy().reshape(2, H, W, 4)
    e = rel_err(got, gold["trace"])
    assert e.ok(), str(e)
    gi.close()
