"""Generate the golden fixture tests/golden/small_scene.npz from the FP64 oracle.

The fixture pins the oracle (tests/test_golden.py re-runs it on CPU) and is the target of the GPU golden test.
It stores its own inputs (triangles, albedo, light, G-buffer), so the check does not depend on the scene generator
or the rasterizer producing the same bytes on another machine.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED, NTRIS, NOBJ = 7, 600, 8
DIM, LEVELS, RES, W, H = 16, 4, 128, 48, 32


def generate():
    import final184_gb300 as g
    import oracle as o
    from gi_case import clip_matrix

    sc = g.SyntheticScene(SEED, NTRIS, NOBJ)
    tri = sc.tri_xyz.copy()
    albedo = sc.albedo.copy()
    rough = sc.roughness.copy()
    lum = np.array(sc.light.luminance, np.float32)
    ldir = np.array(sc.light.direction, np.float32)
    fo = o.grid_frame(o.make_bounds((-10, -10, -10), (10, 10, 10)), DIM, ldir)
    keys = o.raster(o.frame_matrix(fo), RES, RES, tri)
    sd = o.shadow_depth(keys)
    l0, cnt = o.voxelize(fo, DIM, RES, tri, albedo, o.make_light(lum, ldir), sd)
    chain, _ = o.mip(l0, LEVELS)
    V = g.look_at(sc.eye, sc.target)
    P = g.perspective(59.0, W / H, 0.1, 100.0)
    gk = o.raster(clip_matrix(P, V), W, H, tri)
    dep, nrm, rgh, tid = o.gbuffer_resolve(gk, tri, rough, V)
    out = o.trace(fo, DIM, LEVELS, chain, V, P, W, H, dep, nrm, rgh)
    return dict(tri=tri, albedo=albedo, rough=rough, lum=lum, ldir=ldir, view=V, proj=P, shadow=sd,
                counts=cnt.astype(np.uint16), l0=l0.astype(np.float64), depth=dep, normal=nrm, rough_px=rgh,
                tri_id=tid, trace=out, dims=np.array([DIM, LEVELS, RES, W, H], np.int64))


if __name__ == "__main__":
    d = generate()
    path = os.path.join(HERE, "small_scene.npz")
    np.savez_compressed(path, **d)
    print(path, os.path.getsize(path), "bytes")
