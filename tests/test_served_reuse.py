"""How much of a served request's trace could be reused exactly (CPU, the oracle's FP32 path).

A served request moves 0-5% of a resident scene's objects, re-voxelizes the dirty bricks and rebuilds the mips.
Exact reuse of an earlier request's pixels would be possible only for pixels whose cones sample no voxel that
changed.  The mip chain spreads every change upwards (a moved object changes voxels up to the 2^3 top level), and
a 60-degree diffuse cone reaches the coarse levels within a few steps, so almost no pixel escapes.  Counted here on
a served scene (128^3 grid, 100k triangles, 400 objects) for the same camera traced before and after the move,
with the moved geometry's G-buffer on both sides (the most favourable case: the served stream's cameras differ per
request, which leaves nothing to reuse at all): the fraction of pixels whose diffuse and specular outputs are
bit-identical is the ceiling of exact reuse.
"""
import numpy as np
import pytest

import oracle as o
from oracle import scene_host

DIM, LEVELS, RES, W, H = 128, 7, 2048, 320, 180


def _chain(sc, tri):
    b = sc.bounds
    fo = o.grid_frame(o.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), DIM,
                      np.array(sc.light.direction, np.float32))
    sd = o.shadow_depth(o.raster(o.frame_matrix(fo), RES, RES, tri))
    light = o.make_light(list(sc.light.luminance), list(sc.light.direction))
    l0, _ = o.voxelize(fo, DIM, RES, tri, sc.albedo, light, sd, f64=False)
    chain, levels = o.mip(l0, LEVELS, f64=False)
    return fo, chain, levels


@pytest.fixture(scope="module")
def scene():
    sc = scene_host.HostScene(4242, 100000, 400)
    return sc, _chain(sc, sc.tri_xyz)


# one object (22-27% of the pixels reusable), four (0-0.2%), 5% of the objects (none)
@pytest.mark.parametrize("nmove,bound", [(1, 0.35), (4, 0.25), (20, 0.01)])
def test_exact_reuse_fraction_after_moves(scene, nmove, bound):
    sc, (fo, chain_a, lv_a) = scene
    rng = np.random.default_rng(5 + nmove)
    tri = sc.tri_xyz.copy()
    for ob in rng.choice(np.arange(1, sc.nobjects), nmove, replace=False):
        f, c = int(sc.object_first[ob]), int(sc.object_count[ob])
        seg = tri[f * 9:(f + c) * 9].reshape(-1, 3)
        seg += rng.uniform(-0.2, 0.2, 3).astype(np.float32)
    _, chain_b, lv_b = _chain(sc, tri)
    changed = [int(np.any(a != b, axis=-1).sum()) for a, b in zip(lv_a, lv_b)]
    assert changed[-1] >= 1  # the change reaches the top level
    worst = 0.0
    for cam in range(2):
        eye, tgt = sc.camera(cam)
        V, P = scene_host.look_at(eye, tgt), scene_host.perspective(59.0, W / H, 0.1, 100.0)
        dep, nrm, rgh, _ = o.gbuffer_resolve(o.raster(P.astype(np.float64) @ V.astype(np.float64), W, H, tri), tri,
                                             sc.roughness, V)
        a = o.trace(fo, DIM, LEVELS, chain_a, V, P, W, H, dep, nrm, rgh, f64=False)
        b = o.trace(fo, DIM, LEVELS, chain_b, V, P, W, H, dep, nrm, rgh, f64=False)
        geo = dep < 1.0
        same = np.all(a == b, axis=-1)
        reusable = float((same[0] & same[1])[geo].mean())
        print("%d object(s) moved, changed voxels per level %s, camera %d: %.2f%% of %d pixels reusable exactly"
              % (nmove, changed, cam, 100 * reusable, int(geo.sum())))
        worst = max(worst, reusable)
    assert worst < bound
