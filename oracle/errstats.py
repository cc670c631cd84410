"""Error statistics of a device result against the FP64 oracle.  TEST INFRASTRUCTURE ONLY.

The parity gate is a TRUE relative error per value, |got - ref| / |ref|, taken over every value above a
near-black floor.  The floor is stated, not tuned: FLOOR_FRAC (1e-3) times the 99th percentile of |ref| over the
nonzero values of the same channel group.  Values at or below the floor are counted, their absolute error is
reported, and a sanity bound holds them within BELOW_FACTOR (2) times the error a value at the floor is allowed
(tol x floor): the FP32 path's absolute noise, ~3e-8 in radiance units on the test scenes, is itself ~1e-3 of the
floor, so the bound at exactly tol x floor would gate rounding noise of near-black pixels.  The groups are the
radiance channels (RGB) and the opacity / occlusion channel (A) of RGBA data, whose scales differ by orders of
magnitude; data whose last axis is not 4 is one group.

Why this floor: below ~1e-3 of the image's bright end a pixel is black on any display (an 8-bit channel steps by
1/255 ~ 3.9e-3 of full scale), and there an FP32 evaluation has a constant ABSOLUTE error of ~1e-8 (the trilinear
weights of a cone sample carry the rounding of its FP32 position, ~3e-5 voxel at 256 voxels), so its relative
error grows without bound as the value goes to zero.  An FP16-stored chain has a bounded RELATIVE error instead.
"""
from typing import NamedTuple

import numpy as np

REL_TOL = 1e-3
FLOOR_FRAC = 1e-3
BELOW_FACTOR = 2.0


class Err(NamedTuple):
    max: float          # max true relative error over the values above the floor
    rms: float          # RMS of the same
    n: int              # values above the floor
    below: int          # values at or below the floor (near-black), not in max / rms
    below_abs: float    # max |got - ref| over those
    below_ratio: float  # max over the groups of (max |got - ref| below the group's floor) / that floor
    floor: float        # the radiance (or single-group) floor
    floor_a: float      # the alpha floor (RGBA data), else 0

    def ok(self, tol=REL_TOL):
        """Every value above its floor within tol relative; every value below it within BELOW_FACTOR x tol x its
        floor."""
        return self.max < tol and self.below_ratio <= BELOW_FACTOR * tol

    @property
    def below_ok(self):
        return self.below_ratio <= BELOW_FACTOR * REL_TOL

    def __str__(self):
        return ("max %.3e rms %.3e over %d values; %d near-black (floor %.2e%s) max abs %.2e (%.2g of the floor)"
                % (self.max, self.rms, self.n, self.below, self.floor,
                   ", alpha floor %.2e" % self.floor_a if self.floor_a else "", self.below_abs, self.below_ratio))


def group_floor(ref, frac=FLOOR_FRAC):
    a = np.abs(np.asarray(ref, dtype=np.float64)).ravel()
    nz = a[a > 0]
    return float(frac * np.percentile(nz, 99)) if nz.size else 0.0


def rel_err(got, ref, frac=FLOOR_FRAC):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    groups = [(got[..., :3], ref[..., :3]), (got[..., 3], ref[..., 3])] if ref.shape and ref.shape[-1] == 4 \
        else [(got, ref)]
    errs, n, below, below_abs, below_ratio, floors = [], 0, 0, 0.0, 0.0, []
    for g, r in groups:
        fl = group_floor(r, frac)
        floors.append(fl)
        d = np.abs(g - r)
        above = np.abs(r) > fl
        e = d[above] / np.abs(r[above])
        errs.append(e)
        n += int(above.sum())
        b = d[~above]
        below += int(b.size)
        if b.size:
            below_abs = max(below_abs, float(b.max()))
            if float(b.max()) > 0.0:
                below_ratio = max(below_ratio, float(b.max()) / fl if fl > 0.0 else float("inf"))
    e = np.concatenate(errs) if errs else np.zeros(0)
    return Err(float(e.max()) if e.size else 0.0, float(np.sqrt(np.mean(e ** 2))) if e.size else 0.0, n, below,
               below_abs, below_ratio, floors[0], floors[1] if len(floors) > 1 else 0.0)
