"""Edge cases of the CUDA path against the oracle (run on a GPU).

- ragged views (1x1, sizes that are not multiples of any warp tile) traced together in one call: each equals the
  same view traced alone, byte for byte, and the oracle within REL_TOL;
- a view with no geometry (every depth at the far plane) traces to exact zeros;
- an empty scene (no triangles, explicit bounds): far shadow map, empty grid, zero image;
- degenerate triangles (repeated vertices, collinear) and triangles partly or wholly outside the grid: shadow map,
  occupancy and counts bit-exact against the oracle;
- cone parameters off the defaults, including diffuse cones narrow enough that their marches run past the
  per-launch schedule table into the device recurrence: within REL_TOL of the oracle;
- views past the size limits (a side over 16384 pixels for the trace, over 8192 for the G-buffer raster) are
  refused on the host with F184GI_ERR_INVALID, before any launch;
- a bounded device wait that expires is reported as F184GI_ERR_TIMEOUT by the next sync, and the context goes on
  working (the failure path of the library's bounded waits, without a GPU fault);
- the smallest grids (16^3, one to four levels; 32^3), FP32 and FP16: counts bit-exact, traces within REL_TOL.
"""
import numpy as np
import pytest

from gi_case import REL_TOL, Case, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(lib):
    c = Case()
    c.voxelize()
    c.mip()
    c.gbuffer()
    return c


@pytest.fixture(scope="module")
def oracle_chain(case, orc):
    fo = case.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), case.res, case.res, case.sc.tri_xyz))
    l0, _ = orc.voxelize(fo, case.dim, case.res, case.sc.tri_xyz, case.sc.albedo, case.oracle_light(), sd)
    chain, _ = orc.mip(l0, case.levels)
    return fo, chain


def make_view(case, W, H):
    """A device G-buffer of the case's camera at W x H and an output buffer."""
    g, torch = case.g, case.torch
    P = g.perspective(59.0, W / H, 0.1, 100.0)
    n = W * H
    bufs = (torch.empty(n, dtype=torch.float32, device=case.dev), torch.empty(n, dtype=torch.int32, device=case.dev),
            torch.empty(n, dtype=torch.int16, device=case.dev), torch.zeros(2 * n * 4, dtype=torch.float32, device=case.dev))
    view = g.make_view(case.V, P, W, H, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr())
    case.gi.gbuffer(case.tri_d.data_ptr(), case.rough_d.data_ptr(), case.ntris, view)
    case.gi.sync()
    return view, P, bufs


def host_gbuffer(bufs, W, H):
    return (bufs[0].cpu().numpy().reshape(H, W), bufs[1].cpu().numpy().view(np.uint32).reshape(H, W),
            bufs[2].cpu().numpy().view(np.uint16).reshape(H, W))


SIZES = [(1, 1), (37, 23), (129, 7), (8, 4), (31, 33)]


def test_ragged_views_one_call_equal_alone_and_oracle(case, orc, oracle_chain):
    fo, chain = oracle_chain
    made = [make_view(case, W, H) for W, H in SIZES]
    case.gi.trace(case.grid, [m[0] for m in made])
    case.gi.sync()
    together = [m[2][3].cpu().numpy().copy() for m in made]
    for (W, H), (view, P, bufs), got in zip(SIZES, made, together):
        bufs[3].zero_()
        case.gi.trace(case.grid, [view])
        case.gi.sync()
        alone = bufs[3].cpu().numpy()
        assert np.array_equal(alone.view(np.uint32), got.view(np.uint32)), (W, H)
        dep, nrm, rgh = host_gbuffer(bufs, W, H)
        ref = orc.trace(fo, case.dim, case.levels, chain, case.V, P, W, H, dep, nrm, rgh)
        e = rel_err(got.reshape(2, H, W, 4), ref)
        assert e.ok(), (W, H, str(e))


def test_view_without_geometry_traces_to_zero(case):
    view, P, bufs = make_view(case, 64, 48)
    bufs[0].fill_(1.0)  # every pixel at the far plane
    bufs[3].fill_(7.0)
    case.gi.trace(case.grid, [view])
    case.gi.sync()
    assert not bufs[3].any()


def test_empty_scene(lib, orc):
    import torch

    import final184_gb300 as g

    dim, levels, res, W, H = 32, 5, 256, 48, 32
    gi = g.VoxelGI(0)
    grid = gi.create_grid(dim, levels, g.FMT_F32, 0, res, g.GRID_KEEP_COUNTS)
    light = g.make_light([4.4, 3.7, 3.2], [0.3, -0.8, 0.2])
    bounds = g.make_bounds((-5, -5, -5), (5, 5, 5))
    dummy = torch.zeros(9, dtype=torch.float32, device="cuda:0")
    gi.voxelize(grid, dummy.data_ptr(), dummy.data_ptr(), 0, light, bounds=bounds)
    gi.mip(grid)
    gi.sync()
    fo = orc.grid_frame(orc.make_bounds((-5, -5, -5), (5, 5, 5)), dim, np.array(light.direction, np.float32))
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), res, res, np.zeros(0, np.float32)))
    assert np.array_equal(gi.read_shadow(grid).view(np.uint32), sd.view(np.uint32))
    assert not gi.read_counts(grid).any()
    for lv in range(levels):
        assert not gi.read_level(grid, lv).any()
    n = W * H
    depth = torch.full((n,), 0.5, dtype=torch.float32, device="cuda:0")
    normal = torch.zeros(n, dtype=torch.int32, device="cuda:0")  # octahedral (0, 0): +z
    rgh = torch.zeros(n, dtype=torch.int16, device="cuda:0")
    out = torch.full((2 * n * 4,), 3.0, dtype=torch.float32, device="cuda:0")
    V = g.look_at([0, 0, 8], [0, 0, 0])
    view = g.make_view(V, g.perspective(59.0, W / H, 0.1, 100.0), W, H, depth.data_ptr(), normal.data_ptr(),
                       rgh.data_ptr(), out.data_ptr())
    gi.trace(grid, [view])
    gi.sync()
    assert not out.any()
    gi.close()


def test_degenerate_and_outside_triangles_bit_exact(lib, orc):
    c = Case(seed=31, ntris=4000, nobj=40, dim=64, levels=6, res=512, width=64, height=36)
    rng = np.random.default_rng(9)
    base = c.sc.tri_xyz.reshape(-1, 3, 3)
    extra = []
    for k in range(300):
        t = base[rng.integers(0, len(base))].copy()
        kind = k % 5
        if kind == 0:
            t[1] = t[0]  # two equal vertices
        elif kind == 1:
            t[2] = 0.5 * (t[0] + t[1])  # collinear
        elif kind == 2:
            t[:] = t[0]  # a point
        elif kind == 3:
            t += np.float32(rng.uniform(8, 30)) * np.sign(rng.normal(size=3)).astype(np.float32)  # partly / wholly out
        else:
            t *= np.float32(3.0)  # stretched across and beyond the grid
        extra.append(t)
    tri = np.concatenate([base, np.asarray(extra, np.float32)]).astype(np.float32).ravel()
    alb = np.concatenate([c.sc.albedo, rng.integers(0, 2 ** 32, len(extra), dtype=np.uint64).astype(np.uint32)])
    c.upload(tri, alb)
    c.voxelize()
    fo = c.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), c.res, c.res, tri))
    assert np.array_equal(c.gi.read_shadow(c.grid).view(np.uint32), sd.view(np.uint32))
    l0, cnt = orc.voxelize(fo, c.dim, c.res, tri, alb, c.oracle_light(), sd)
    assert np.array_equal(c.gi.read_counts(c.grid), cnt.astype(np.uint32))
    got = c.gi.read_level(c.grid, 0)
    assert np.array_equal(got[..., 3] > 0, l0[..., 3] > 0)
    e = rel_err(got, l0)
    assert e.ok(), str(e)


@pytest.mark.parametrize("kw", [
    dict(diffuse_tan_half=0.08),  # narrow diffuse cones: ~50 steps, past the 24-step schedule table
    dict(diffuse_cones=1, specular=0),
    dict(max_distance=20.0, step_factor=1.0, start_offset=2.0),
    dict(diffuse_tilt_deg=30.0, min_spec_tan_half=0.2),
])
def test_cone_parameters_against_oracle(case, orc, oracle_chain, kw):
    import final184_gb300 as g

    fo, chain = oracle_chain
    p = g.default_cone_params()
    q = orc.default_params()
    for k, v in kw.items():
        setattr(p, k, v)
        setattr(q, k, v)
    got = case.trace(p)
    dep, nrm, rgh, _ = case.gbuffer_host()
    ref = orc.trace(fo, case.dim, case.levels, chain, case.V, case.P, case.W, case.H, dep, nrm, rgh, params=q)
    e = rel_err(got, ref)
    print(kw, e)
    assert e.ok(), str(e)
    if kw.get("specular", 1) == 0:
        assert not got[1].any()


def test_expired_bounded_wait_is_reported_and_the_context_stays_usable(case):
    from final184_gb300 import _abi

    before = case.trace().copy()
    case.gi.selftest_bounded_wait(1000, complete=True)
    case.gi.sync()  # a completed wait leaves no status
    case.gi.selftest_bounded_wait(1000, complete=False)
    with pytest.raises(_abi.F184Error) as err:
        case.gi.sync()
    assert err.value.code == _abi.ERR_TIMEOUT and "bounded device wait" in str(err.value)
    case.gi.sync()  # the status was consumed by the report
    after = case.trace()
    assert np.array_equal(before.view(np.uint32), after.view(np.uint32))


def test_expired_copy_wait_retires_the_context(lib):
    """An expired wait on a bulk copy (as the mip pass records one; the self-test's wait involves no copy) makes
    the context refuse every later call, since such a copy may still be landing in shared memory."""
    import final184_gb300 as g

    c = Case(ntris=3000, nobj=30, dim=32, levels=5, res=256, width=64, height=32)
    c.voxelize()
    c.gi.selftest_bounded_wait(1000, complete=False, as_copy_wait=True)
    with pytest.raises(g.F184Error) as err:
        c.gi.sync()
    assert err.value.code == g._abi.ERR_TIMEOUT and "bulk copy" in str(err.value)
    for call in (lambda: c.gi.mip(c.grid), lambda: c.gi.trace(c.grid, [c.view]),
                 lambda: c.gi.voxelize(c.grid, c.tri_d.data_ptr(), c.alb_d.data_ptr(), c.ntris, c.sc.light,
                                       bounds=c.sc.bounds)):
        with pytest.raises(g.F184Error) as err:
            call()
        assert err.value.code == g._abi.ERR_TIMEOUT
    c.gi.close()
    fresh = Case(ntris=3000, nobj=30, dim=32, levels=5, res=256, width=64, height=32)
    fresh.voxelize()  # a new context works
    fresh.mip()


def test_oversize_views_are_refused_before_any_launch(case):
    import final184_gb300 as g
    from final184_gb300 import _abi

    view, P, bufs = make_view(case, 8, 4)
    for W, H in [(16385, 1), (1, 16385)]:  # past both limits
        big = g.make_view(case.V, P, W, H, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(),
                          bufs[3].data_ptr())
        with pytest.raises(_abi.F184Error) as err:
            case.gi.trace(case.grid, [big])
        assert err.value.code == _abi.ERR_INVALID and "16384" in str(err.value)
        with pytest.raises(_abi.F184Error) as err:
            case.gi.gbuffer(case.tri_d.data_ptr(), case.rough_d.data_ptr(), case.ntris, big)
        assert err.value.code == _abi.ERR_INVALID
    # past the raster's limit only: the G-buffer call refuses it (the view is never traced: its buffers are small)
    wide = g.make_view(case.V, P, 8193, 1, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(),
                       bufs[3].data_ptr())
    with pytest.raises(_abi.F184Error) as err:
        case.gi.gbuffer(case.tri_d.data_ptr(), case.rough_d.data_ptr(), case.ntris, wide)
    assert err.value.code == _abi.ERR_INVALID and "8192" in str(err.value)
    case.gi.sync()  # nothing was launched: no device status


def test_non_finite_triangles_skipped_and_reported(lib, orc):
    """Malformed triangle buffers: triangles with a NaN or infinite coordinate are skipped by the shadow raster, the
    voxelizer and the G-buffer raster (as by the oracle), and the next sync reports F184GI_ERR_INVALID; the shadow
    map, occupancy, counts and the G-buffer stay bit-exact.  The server refuses such a scene up front."""
    import final184_gb300 as g

    c = Case(ntris=5000, nobj=40, dim=32, levels=5, res=256, width=96, height=64)
    tri = c.sc.tri_xyz.copy().reshape(-1, 9)
    rng = np.random.default_rng(11)
    bad = rng.choice(np.arange(12, len(tri)), 60, replace=False)
    vals = np.array([np.nan, np.inf, -np.inf], np.float32)
    for k, t in enumerate(bad):
        tri[t, rng.integers(0, 9)] = vals[k % 3]
    tri = tri.ravel()
    c.upload(tri, c.sc.albedo)
    c.gi.voxelize(c.grid, c.tri_d.data_ptr(), c.alb_d.data_ptr(), c.ntris, c.sc.light, bounds=c.sc.bounds)
    with pytest.raises(g.F184Error) as e:
        c.gi.sync()
    assert e.value.code == g._abi.ERR_INVALID and "NaN or infinite" in str(e.value)
    fo = c.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), c.res, c.res, tri))
    assert np.array_equal(c.gi.read_shadow(c.grid).view(np.uint32), sd.view(np.uint32))
    _, cnt = orc.voxelize(fo, c.dim, c.res, tri, c.sc.albedo, c.oracle_light(), sd)
    assert np.array_equal(c.gi.read_counts(c.grid), cnt.astype(np.uint32))
    c.gi.gbuffer(c.tri_d.data_ptr(), c.rough_d.data_ptr(), c.ntris, c.view, c.tri_id.data_ptr())
    with pytest.raises(g.F184Error):
        c.gi.sync()
    from gi_case import clip_matrix

    keys = orc.raster(clip_matrix(c.P, c.V), c.W, c.H, tri)
    dep, _, _, tid = orc.gbuffer_resolve(keys, tri, c.sc.roughness, c.V)
    gd, _, _, gt = c.gbuffer_host()
    assert np.array_equal(gt, tid) and np.array_equal(gd.view(np.uint32), dep.view(np.uint32))
    c.gi.sync()  # the status was consumed: the context keeps working
    srv = g.Server(0)
    with pytest.raises(g.F184Error) as e:
        srv.add_scene(0, g.GridDesc(32, 5, g.FMT_F16, 0, 256, 0), tri, c.sc.albedo, c.sc.bounds, c.sc.light)
    assert e.value.code == g._abi.ERR_INVALID
    srv.close()


@pytest.mark.parametrize("dim,levels,fmt", [(16, 1, 0), (16, 4, 0), (16, 4, 1), (32, 5, 1)])
def test_tiny_grids_against_oracle(lib, orc, dim, levels, fmt):
    """The smallest grids (16^3: eight 8^3 bricks, the coarsest level 2^3), with one level (no quadrilinear blend
    at all) up to the full chain, FP32 and FP16: occupancy and counts bit-exact, the traced view within REL_TOL of
    the oracle."""
    c = Case(ntris=4000, nobj=30, dim=dim, levels=levels, res=128, width=96, height=64, fmt=fmt)
    c.voxelize()
    c.mip()
    c.gbuffer()
    got = c.trace()
    fo = c.oracle_frame()
    sd = orc.shadow_depth(orc.raster(orc.frame_matrix(fo), c.res, c.res, c.sc.tri_xyz))
    l0, cnt = orc.voxelize(fo, dim, c.res, c.sc.tri_xyz, c.sc.albedo, c.oracle_light(), sd)
    assert np.array_equal(c.gi.read_counts(c.grid), cnt)
    chain, _ = orc.mip(l0, levels)
    dep, nrm, rgh, _ = c.gbuffer_host()
    ref = orc.trace(fo, dim, levels, chain, c.V, c.P, c.W, c.H, dep, nrm, rgh)
    assert ref[0, ..., :3].max() > 0
    e = rel_err(got, ref)
    print("dim %d, %d level(s), %s:" % (dim, levels, "FP16" if fmt else "FP32"), e)
    assert e.ok(), str(e)
