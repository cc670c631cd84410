"""Shared set-up for GPU parity tests: one seeded scene run through the CUDA path and the CPU oracle.

Tolerance used throughout (oracle/errstats.py): TRUE relative error |gpu - oracle| / |oracle| per value, below
REL_TOL = 1e-3 over every value above the near-black floor (1e-3 of the 99th percentile of the nonzero |oracle|
values of its channel group: radiance RGB, opacity A); values at or below the floor are counted and their
absolute error must stay below twice REL_TOL times the floor (oracle/errstats.py says why).
"""
import numpy as np

from oracle.errstats import FLOOR_FRAC, REL_TOL, Err, rel_err  # noqa: F401


def clip_matrix(proj, view):
    """proj * view in FP64 in the operation order f184gi_gbuffer uses (products rounded, summed j = 0..3)."""
    P = np.asarray(proj, dtype=np.float32).reshape(4, 4)
    V = np.asarray(view, dtype=np.float32).reshape(4, 4)
    M = np.zeros((4, 4), dtype=np.float64)
    for r in range(4):
        for k in range(4):
            acc = 0.0
            for j in range(4):
                acc += float(P[r, j]) * float(V[j, k])
            M[r, k] = acc
    return M


class Case:
    """scene -> device buffers -> (voxelize, mip, gbuffer, trace) on the GPU, with oracle counterparts."""

    def __init__(self, seed=184, ntris=20000, nobj=200, dim=64, levels=6, res=1024, width=320, height=180,
                 fmt=0, keep_counts=True, aniso=False):
        import torch

        import final184_gb300 as g

        self.g = g
        self.torch = torch
        self.dev = torch.device("cuda:0")
        self.sc = g.SyntheticScene(seed, ntris, nobj)
        self.dim, self.levels, self.res, self.W, self.H, self.fmt = dim, levels, res, width, height, fmt
        self.gi = g.VoxelGI(0)
        self.aniso = aniso
        self.grid = self.gi.create_grid(dim, levels, fmt, 1 if aniso else 0, res,
                                        g.GRID_KEEP_COUNTS if keep_counts else 0)
        self.upload(self.sc.tri_xyz, self.sc.albedo)
        self.rough_d = torch.from_numpy(self.sc.roughness).to(self.dev)
        self.V = g.look_at(self.sc.eye, self.sc.target)
        self.P = g.perspective(59.0, width / height, 0.1, 100.0)
        n = width * height
        self.depth = torch.empty(n, dtype=torch.float32, device=self.dev)
        self.normal = torch.empty(n, dtype=torch.int32, device=self.dev)
        self.rgh = torch.empty(n, dtype=torch.int16, device=self.dev)
        self.tri_id = torch.empty(n, dtype=torch.int32, device=self.dev)
        self.out = torch.empty(2 * n * 4, dtype=torch.float32, device=self.dev)
        self.view = g.make_view(self.V, self.P, width, height, self.depth.data_ptr(), self.normal.data_ptr(),
                                self.rgh.data_ptr(), self.out.data_ptr())

    def upload(self, tri, albedo):
        torch = self.torch
        self.tri_d = torch.from_numpy(np.ascontiguousarray(tri, dtype=np.float32)).to(self.dev)
        self.alb_d = torch.from_numpy(np.ascontiguousarray(albedo, dtype=np.uint32).view(np.int32)).to(self.dev)
        self.ntris = self.tri_d.numel() // 9

    def voxelize(self, bounds=True, dirty=None):
        dptr, nd = None, 0
        if dirty is not None:
            self.dirty_d = self.torch.from_numpy(np.asarray(dirty, dtype=np.uint32).view(np.int32)).to(self.dev)
            dptr, nd = self.dirty_d.data_ptr(), len(dirty)
        self.gi.voxelize(self.grid, self.tri_d.data_ptr(), self.alb_d.data_ptr(), self.ntris, self.sc.light,
                         bounds=self.sc.bounds if bounds else None, dirty_ptr=dptr, ndirty=nd)
        self.gi.sync()

    def mip(self):
        self.gi.mip(self.grid)
        self.gi.sync()

    def gbuffer(self):
        self.gi.gbuffer(self.tri_d.data_ptr(), self.rough_d.data_ptr(), self.ntris, self.view, self.tri_id.data_ptr())
        self.gi.sync()

    def trace(self, params=None):
        self.gi.trace(self.grid, [self.view], params)
        self.gi.sync()
        return self.out.cpu().numpy().reshape(2, self.H, self.W, 4)

    def gbuffer_host(self):
        H, W = self.H, self.W
        return (self.depth.cpu().numpy().reshape(H, W), self.normal.cpu().numpy().view(np.uint32).reshape(H, W),
                self.rgh.cpu().numpy().view(np.uint16).reshape(H, W),
                self.tri_id.cpu().numpy().view(np.uint32).reshape(H, W))

    # ---- oracle side ----
    def oracle_frame(self):
        import oracle as o

        ld = np.array(self.sc.light.direction, np.float32)
        b = self.sc.bounds
        return o.grid_frame(o.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), self.dim, ld)

    def oracle_light(self):
        import oracle as o

        return o.make_light(list(self.sc.light.luminance), list(self.sc.light.direction))
