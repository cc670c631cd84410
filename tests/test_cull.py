"""View culling in the C++ adapter (include/f184gi_foreground.hpp) against the reference's own Math library compiled
from source: Frustum::Transformed / UpdatePlanes, BoundingBox::Transformed and Frustum::IsInsideFast bit for bit,
Frustum::Define(projection) to rounding (the adapter inverts the projection in FP64), and CullList's decisions on
whole (matrix, primitive) lists.  CPU only."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def ref(orc):
    r = orc.ref_lib()
    if r is None:
        pytest.skip("reference sources not present on this machine")
    return r


@pytest.fixture(scope="module")
def cull(lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cull") / "libcull.so")
    libdir = os.path.join(ROOT, "final184_gb300")
    # -ffp-contract=off: the adapter's arithmetic rounds each operation, as the reference's scalar code does
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "cull_shim.cpp"), "-o", out,
                    "-L", libdir, "-lf184gi", "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    c = C.CDLL(out)
    V = C.c_void_p
    c.cull_define.argtypes = [V, V]
    c.cull_transformed.argtypes = [V, V, V]
    c.cull_bounds_transformed.argtypes = [V, V, V, V]
    c.cull_inside_fast.argtypes = [V, V, V]
    c.cull_list.argtypes = [V, C.c_uint32, V, V, V]
    return c


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def trs(ref, rng, mirror=False):
    """A tc::Matrix3x4 from translation, a random unit quaternion and a scale (one axis negative when mirror)."""
    t = rng.uniform(-10, 10, 3).astype(np.float32)
    q = rng.normal(size=4)
    q = (q / np.linalg.norm(q)).astype(np.float32)
    s = rng.uniform(0.3, 3.0, 3).astype(np.float32)
    if mirror:
        s[rng.integers(0, 3)] *= -1
    m = np.zeros(12, np.float32)
    ref.ref_matrix_trs(p(t), p(q), p(s), p(m))
    return m


def ref_frustum(ref, g, rng):
    near, far = float(rng.uniform(0.05, 1.0)), float(rng.uniform(20, 200))
    proj = g.perspective(float(rng.uniform(30, 100)), float(rng.uniform(0.5, 2.5)), near, far)
    proj = np.ascontiguousarray(proj.astype(np.float32).ravel())
    f = np.zeros(66, np.float32)
    ref.ref_frustum_define(p(proj), p(f))
    ref_frustum.ratio = far / near
    return proj, f


def random_boxes(rng, n, spread=30.0):
    c = rng.uniform(-spread, spread, (n, 3))
    h = rng.uniform(0.01, 4.0, (n, 3))
    return np.ascontiguousarray(np.concatenate([c - h, c + h], 1).astype(np.float32))


def test_define_from_projection_matches_to_rounding(ref, cull):
    import final184_gb300 as g

    rng = np.random.default_rng(11)
    for _ in range(50):
        proj, want = ref_frustum(ref, g, rng)
        got = np.zeros(66, np.float32)
        assert cull.cull_define(p(proj), p(got)) == 0
        # inverting an FP32 projection loses about far/near ulps on the far corners, in the reference's FP32
        # inverse and in this FP64 one alike (both measured at up to ~5e-5 of the far corners against an exact
        # inverse at far/near ~ 1700): the tolerance follows that ratio
        tol = 1e-5 + 1.2e-7 * ref_frustum.ratio
        wv, gv = want[42:].reshape(8, 3), got[42:].reshape(8, 3)
        scale = np.abs(wv).max()
        assert np.abs(gv - wv).max() <= tol * scale
        wp, gp = want[:42].reshape(6, 7), got[:42].reshape(6, 7)
        assert np.abs(gp[:, :6] - wp[:, :6]).max() <= tol  # unit normals and their absolute values
        assert np.abs(gp[:, 6] - wp[:, 6]).max() <= tol * scale


def test_transformed_frustum_bit_exact(ref, cull):
    import final184_gb300 as g

    rng = np.random.default_rng(12)
    flips = 0
    for k in range(200):
        _, f = ref_frustum(ref, g, rng)
        m = trs(ref, rng, mirror=(k % 4 == 3))
        want, got = np.zeros(66, np.float32), np.zeros(66, np.float32)
        ref.ref_frustum_transformed(p(f), p(m), p(want))
        cull.cull_transformed(p(f), p(m), p(got))
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), k
        # the inner side of the near plane holds the far corners, mirrored or not (the flip in UpdatePlanes)
        n, d = got[0:3], got[6]
        flips += k % 4 == 3
        assert float(n @ got[42 + 15:45 + 15]) + float(d) > 0
    assert flips == 50


def test_bounds_transformed_bit_exact(ref, cull):
    rng = np.random.default_rng(13)
    boxes = random_boxes(rng, 500)
    for i, b in enumerate(boxes):
        m = trs(ref, rng, mirror=(i % 3 == 0))
        mn, mx = np.ascontiguousarray(b[:3]), np.ascontiguousarray(b[3:])
        want, got = np.zeros(6, np.float32), np.zeros(6, np.float32)
        ref.ref_bbox_transformed(p(mn), p(mx), p(m), p(want))
        cull.cull_bounds_transformed(p(mn), p(mx), p(m), p(got))
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i


def test_inside_fast_decisions_identical(ref, cull):
    import final184_gb300 as g

    rng = np.random.default_rng(14)
    counts = {0: 0, 2: 0}
    for _ in range(10):
        _, f0 = ref_frustum(ref, g, rng)
        f = np.zeros(66, np.float32)
        ref.ref_frustum_transformed(p(f0), p(trs(ref, rng)), p(f))
        for b in random_boxes(rng, 2000, spread=60.0):
            mn, mx = np.ascontiguousarray(b[:3]), np.ascontiguousarray(b[3:])
            want = ref.ref_frustum_inside_fast(p(f), p(mn), p(mx))
            assert cull.cull_inside_fast(p(f), p(mn), p(mx)) == want
            counts[want] += 1
    assert min(counts.values()) > 2000, counts  # both answers well represented


def test_cull_list_keeps_the_reference_pairs(ref, cull):
    import final184_gb300 as g

    rng = np.random.default_rng(15)
    n = 3000
    _, f0 = ref_frustum(ref, g, rng)
    f = np.zeros(66, np.float32)
    ref.ref_frustum_transformed(p(f0), p(trs(ref, rng)), p(f))
    boxes = random_boxes(rng, n, spread=8.0)
    mats = np.ascontiguousarray(np.stack([trs(ref, rng, mirror=(i % 5 == 0)) for i in range(n)]))
    keep = np.zeros(n, np.uint8)
    cull.cull_list(p(f), n, p(mats), p(boxes), p(keep))
    want = np.zeros(n, np.uint8)
    for i in range(n):
        wb = np.zeros(6, np.float32)
        mn, mx, m = boxes[i, :3].copy(), boxes[i, 3:].copy(), mats[i].copy()  # held by name across the calls
        ref.ref_bbox_transformed(p(mn), p(mx), p(m), p(wb))
        wmn, wmx = wb[:3].copy(), wb[3:].copy()
        want[i] = ref.ref_frustum_inside_fast(p(f), p(wmn), p(wmx)) != 0
    assert np.array_equal(keep, want)
    assert 0 < keep.sum() < n
