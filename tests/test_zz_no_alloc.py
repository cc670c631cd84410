"""f184gi_gbuffer_static: the G-buffer raster on a fixed device array, against f184gi_gbuffer.

Collected last on purpose, and correct both alone in a fresh process and after every other test: the first call
on the device does the array's set-up.  Two calls in a row on one stream, with different meshes and camera sizes,
must each give the same G-buffer as f184gi_gbuffer (bit-exact, like every G-buffer test) and leave the context's
device memory untouched.
"""
import ctypes as C

import numpy as np
import pytest


def _gbuffer_case(g, torch, seed, ntris, nobj, W, H, cam):
    sc = g.SyntheticScene(seed, ntris, nobj)
    dev = torch.device("cuda:0")
    eye, tgt = sc.camera(cam)
    V, P = g.look_at(eye, tgt), g.perspective(59.0, W / H, 0.1, 100.0)
    return dict(sc=sc, tri=torch.from_numpy(sc.tri_xyz).to(dev), rough=torch.from_numpy(sc.roughness).to(dev),
                V=V, P=P, W=W, H=H)


def _planes(torch, case):
    n = case["W"] * case["H"]
    dev = torch.device("cuda:0")
    return (torch.full((n,), -1.0, dtype=torch.float32, device=dev), torch.zeros(n, dtype=torch.int32, device=dev),
            torch.zeros(n, dtype=torch.int16, device=dev), torch.zeros(n, dtype=torch.int32, device=dev))


def _view(g, case, planes):
    d, nr, rg, _ = planes
    return g.make_view(case["V"], case["P"], case["W"], case["H"], d.data_ptr(), nr.data_ptr(), rg.data_ptr(), 0)


@pytest.mark.gpu
def test_static_scratch_gbuffer_matches_gbuffer_twice_in_a_row(lib):
    import torch

    import final184_gb300 as g

    cases = [_gbuffer_case(g, torch, 31, 20000, 200, 640, 360, 0),
             _gbuffer_case(g, torch, 32, 200000, 800, 1920, 1080, 1)]
    # the existing entry point, on its own context
    ref_ctx = g.VoxelGI(0)
    ref = []
    for cs in cases:
        pl = _planes(torch, cs)
        v = _view(g, cs, pl)
        ref_ctx.gbuffer(cs["tri"].data_ptr(), cs["rough"].data_ptr(), cs["sc"].ntris, v, tri_id_ptr=pl[3].data_ptr())
        ref.append(pl)
    ref_ctx.sync()
    # the static-scratch entry point: both calls back to back on one stream, through the C ABI
    gi = g.VoxelGI(0)
    used0 = gi.memory_used()
    got = []
    stream = torch.cuda.Stream()
    planes = [_planes(torch, cs) for cs in cases]
    torch.cuda.synchronize()  # the planes are initialised on torch's stream
    free = []
    for cs, pl in zip(cases, planes):
        v = _view(g, cs, pl)
        free.append(torch.cuda.mem_get_info()[0])
        g.check(gi.lib.f184gi_gbuffer_static(gi.ctx, cs["tri"].data_ptr(), cs["rough"].data_ptr(), cs["sc"].ntris,
                                             C.byref(v), C.c_void_p(pl[3].data_ptr()),
                                             C.c_void_p(stream.cuda_stream)))
        got.append(pl)
    gi.sync(stream.cuda_stream)
    free.append(torch.cuda.mem_get_info()[0])
    assert gi.memory_used() == used0  # nothing was allocated on the context
    # nor on the device: after the first call (which may load the module holding the array), the second call
    # leaves the device's free memory as it was
    assert free[2] == free[1], (free[1], free[2])
    for a, b in zip(ref, got):
        for x, y in zip(a, b):
            assert torch.equal(x.view(torch.int32) if x.dtype == torch.float32 else x,
                               y.view(torch.int32) if y.dtype == torch.float32 else y)
        assert int((b[0] > 0).sum()) > 0  # the camera saw geometry
    ref_ctx.close()
    gi.close()


@pytest.mark.gpu
def test_static_scratch_gbuffer_rejects_sizes_beyond_its_limit(lib):
    import torch

    import final184_gb300 as g

    gi = g.VoxelGI(0)
    cs = _gbuffer_case(g, torch, 33, 2000, 20, 64, 64, 0)
    pl = _planes(torch, cs)
    v = _view(g, cs, pl)
    with pytest.raises(g.F184Error) as e:
        g.check(gi.lib.f184gi_gbuffer_static(gi.ctx, cs["tri"].data_ptr(), cs["rough"].data_ptr(), 262145,
                                             C.byref(v), None, None))
    assert e.value.code == g._abi.ERR_INVALID and "262144" in str(e.value)
    big = g.make_view(cs["V"], cs["P"], 2048, 1025, pl[0].data_ptr(), pl[1].data_ptr(), pl[2].data_ptr(), 0)
    with pytest.raises(g.F184Error) as e:
        g.check(gi.lib.f184gi_gbuffer_static(gi.ctx, cs["tri"].data_ptr(), cs["rough"].data_ptr(), cs["sc"].ntris,
                                             C.byref(big), None, None))
    assert e.value.code == g._abi.ERR_INVALID and "2097152" in str(e.value)
    gi.close()
