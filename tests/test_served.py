"""The served form (f184gi_server_*): continuous batching over device-resident scenes.

GPU: every request's traced output is byte-identical whether it ran alone or batched with others; dirty-brick
re-voxelization after moves equals a full voxelization of the moved scene; host-buffer requests equal device-buffer
requests; admission against the HBM budget, cancellation and bounded waits.  CPU: creating a server without a
GPU fails with a status code (no fallback).
"""
import numpy as np
import pytest

SEEDS = [11, 12, 13]


def test_server_needs_a_gpu(lib):
    import torch

    import final184_gb300 as g

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(g.F184Error):
        g.Server(0)


class Fixture:
    """Three seeded scenes, device G-buffers for a few views each, and a reproducible request list."""

    def __init__(self, dim=64, levels=6, res=1024, fmt=1):
        import torch

        import final184_gb300 as g

        self.g, self.torch = g, torch
        self.dev = torch.device("cuda:0")
        self.scenes = [g.SyntheticScene(s, 20000, 200) for s in SEEDS]
        self.desc = g.GridDesc(dim, levels, fmt, 0, res, 0)
        gi = g.VoxelGI(0)
        self.views = {}  # (scene, view) -> (V, P, W, H, depth, normal, rough)
        sizes = [(160, 90), (128, 128), (200, 120), (96, 64)]
        for si, sc in enumerate(self.scenes):
            tri = torch.from_numpy(sc.tri_xyz).to(self.dev)
            rough = torch.from_numpy(sc.roughness).to(self.dev)
            for vi, (W, H) in enumerate(sizes):
                eye, tgt = sc.camera(vi)
                V = g.look_at(eye, tgt)
                P = g.perspective(59.0, W / H, 0.1, 100.0)
                n = W * H
                d = torch.empty(n, dtype=torch.float32, device=self.dev)
                nr = torch.empty(n, dtype=torch.int32, device=self.dev)
                rg = torch.empty(n, dtype=torch.int16, device=self.dev)
                out = torch.empty(2 * n * 4, dtype=torch.float32, device=self.dev)
                view = g.make_view(V, P, W, H, d.data_ptr(), nr.data_ptr(), rg.data_ptr(), out.data_ptr())
                gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view)
                self.views[(si, vi)] = (V, P, W, H, d, nr, rg)
        gi.sync()
        gi.close()
        rng = np.random.default_rng(5)
        self.requests = []  # (scene, [view ids], [moves])
        for k in range(12):
            si = int(rng.integers(0, 3))
            nv = int(rng.integers(1, 5))
            vids = [int(x) for x in rng.choice(4, nv, replace=False)]
            sc = self.scenes[si]
            moves = []
            for o in rng.choice(np.arange(1, sc.nobjects), 3, replace=False):
                off = rng.uniform(-0.3, 0.3, 3).astype(np.float32)
                moves.append((int(sc.object_first[o]), int(sc.object_count[o]), [float(x) for x in off]))
            self.requests.append((si, vids, moves))

    def server(self, **kw):
        srv = self.g.Server(0, **kw)
        for si, sc in enumerate(self.scenes):
            srv.add_scene(si, self.desc, sc.tri_xyz, sc.albedo, sc.bounds, sc.light)
        return srv

    def make_views(self, si, vids, out_dtype=np.float32):
        outs, views = [], []
        for vi in vids:
            V, P, W, H, d, nr, rg = self.views[(si, vi)]
            out = self.torch.zeros(2 * W * H * 4, dtype=self.torch.float32, device=self.dev)
            outs.append(out)
            views.append(self.g.make_view(V, P, W, H, d.data_ptr(), nr.data_ptr(), rg.data_ptr(), out.data_ptr()))
        return views, outs


@pytest.fixture(scope="module")
def fx(lib):
    return Fixture()


def run_all(fx, srv, one_at_a_time):
    results, keep = [], []
    tickets = []
    for si, vids, moves in fx.requests:
        views, outs = fx.make_views(si, vids)
        keep.append(outs)
        t = srv.submit(si, views, moves)
        tickets.append(t)
        if one_at_a_time:
            srv.wait(t)
    res = [srv.wait(t) for t in tickets]
    fx.torch.cuda.synchronize()
    for outs in keep:
        results.append([o.cpu().numpy().copy() for o in outs])
    return results, res


@pytest.mark.gpu
def test_each_request_same_alone_and_in_the_mix(fx):
    srv = fx.server(slots=2, max_batch_views=32)
    alone, _ = run_all(fx, srv, one_at_a_time=True)
    srv.close()
    srv = fx.server(slots=2, max_batch_views=32)
    mixed, res = run_all(fx, srv, one_at_a_time=False)
    st = srv.stats()
    srv.close()
    assert st.requests_done == len(fx.requests)
    assert max(r.batch for r in res) < len(fx.requests)  # some requests really shared a batch
    for a, b in zip(alone, mixed):
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert any(float(np.abs(x).sum()) > 0 for a in mixed for x in a)


@pytest.mark.gpu
def test_concurrent_submitters_match_alone(fx):
    """One host thread per scene submits that scene's requests (in order) while the others submit theirs: every
    result equals the same request run alone."""
    import threading

    srv = fx.server(slots=2, max_batch_views=32)
    alone, _ = run_all(fx, srv, one_at_a_time=True)
    srv.close()
    srv = fx.server(slots=3, max_batch_views=32)
    tickets, keep = [None] * len(fx.requests), [None] * len(fx.requests)

    def submitter(scene):
        for i, (si, vids, moves) in enumerate(fx.requests):
            if si == scene:
                views, outs = fx.make_views(si, vids)
                keep[i] = outs
                tickets[i] = srv.submit(si, views, moves)

    threads = [threading.Thread(target=submitter, args=(k,)) for k in range(len(fx.scenes))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for tk in tickets:
        assert srv.wait(tk).status == 0
    fx.torch.cuda.synchronize()
    srv.close()
    for a, outs in zip(alone, keep):
        for x, y in zip(a, outs):
            assert np.array_equal(x.view(np.uint32), y.cpu().numpy().view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("slots", [2, 4])
def test_same_scene_requests_pipelined_in_order(fx, slots):
    """Requests of one scene submitted at once run one per batch in order, each batch's update of the scene
    waiting on the previous batch (another slot) instead of the scene blocking admission: every result equals the
    same request run alone, after the moves of the requests before it."""
    sc = fx.scenes[0]
    rng = np.random.default_rng(17)
    reqs = []  # every request on scene 0, each moving three of its objects
    for _, vids, _ in fx.requests:
        moves = [(int(sc.object_first[o]), int(sc.object_count[o]),
                  [float(x) for x in rng.uniform(-0.3, 0.3, 3).astype(np.float32)])
                 for o in rng.choice(np.arange(1, sc.nobjects), 3, replace=False)]
        reqs.append((0, vids, moves))
    srv = fx.server(slots=2, max_batch_views=32)
    alone = []
    for si, vids, moves in reqs:
        views, outs = fx.make_views(si, vids)
        assert srv.wait(srv.submit(si, views, moves)).status == 0
        fx.torch.cuda.synchronize()
        alone.append([o.cpu().numpy().copy() for o in outs])
    srv.close()
    srv = fx.server(slots=slots, max_batch_views=32)
    keep, tickets = [], []
    for si, vids, moves in reqs:
        views, outs = fx.make_views(si, vids)
        keep.append(outs)
        tickets.append(srv.submit(si, views, moves))
    res = [srv.wait(t) for t in tickets]
    fx.torch.cuda.synchronize()
    srv.close()
    assert all(r.status == 0 for r in res)
    batches = [r.batch for r in res]
    assert batches == sorted(batches) and len(set(batches)) == len(batches)  # one per batch, in order
    for a, outs in zip(alone, keep):
        for x, y in zip(a, outs):
            assert np.array_equal(x.view(np.uint32), y.cpu().numpy().view(np.uint32))


@pytest.mark.gpu
def test_dirty_updates_equal_full_voxelization(fx):
    g, torch = fx.g, fx.torch
    srv = fx.server(slots=1)
    # apply every request's moves of scene 0 in order, then trace view 0
    moved = g.SyntheticScene(SEEDS[0], 20000, 200)
    tri = moved.tri_xyz.copy()
    for si, vids, moves in fx.requests:
        if si != 0:
            continue
        views, outs = fx.make_views(0, [0])
        srv.wait(srv.submit(0, views, moves))
        for f, c, off in moves:
            seg = tri[f * 9:(f + c) * 9].reshape(-1, 3)
            seg += np.asarray(off, dtype=np.float32)
            tri[f * 9:(f + c) * 9] = seg.ravel()
    views, served_out = fx.make_views(0, [0])
    srv.wait(srv.submit(0, views, []))
    srv.close()
    # the same geometry voxelized from scratch through the plain API
    gi = g.VoxelGI(0)
    grid = gi.create_grid(fx.desc.dim, fx.desc.levels, fx.desc.format, 0, fx.desc.shadow_res)
    td = torch.from_numpy(tri).to(fx.dev)
    ad = torch.from_numpy(moved.albedo.view(np.int32)).to(fx.dev)
    gi.voxelize(grid, td.data_ptr(), ad.data_ptr(), moved.ntris, moved.light, bounds=moved.bounds)
    gi.mip(grid)
    views2, plain_out = fx.make_views(0, [0])
    gi.trace(grid, views2)
    gi.sync()
    a = served_out[0].cpu().numpy()
    b = plain_out[0].cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    gi.close()


@pytest.fixture(scope="module")
def fx32(lib):
    return Fixture(fmt=0)


@pytest.mark.gpu
def test_every_trace_variant_matches_the_plain_path_fp32(fx32):
    """As below on FP32 chains (the plain path's storage)."""
    test_every_trace_variant_matches_the_plain_path(fx32)


@pytest.mark.gpu
def test_every_trace_variant_matches_the_plain_path(fx):
    """Each cone-trace kernel variant (tile shape, CTAs per SM), launched with a warp per tile or as a capped
    persistent wave, gives the plain one-shot launch's bytes."""
    g, torch = fx.g, fx.torch
    si, vids = 2, [0, 1, 2, 3]
    sc = fx.scenes[si]
    gi = g.VoxelGI(0)
    grid = gi.create_grid(fx.desc.dim, fx.desc.levels, fx.desc.format, 0, fx.desc.shadow_res, fx.desc.flags)
    td = torch.from_numpy(sc.tri_xyz).to(fx.dev)
    ad = torch.from_numpy(sc.albedo.view(np.int32)).to(fx.dev)
    gi.voxelize(grid, td.data_ptr(), ad.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
    gi.mip(grid)
    views, plain = fx.make_views(si, vids)
    gi.trace(grid, views)
    gi.sync()
    ref = [o.cpu().numpy() for o in plain]
    gi.close()
    tuned = fx.server(slots=1)
    views, outs = fx.make_views(si, vids)
    tuned.wait(tuned.submit(si, views, []))
    st = tuned.stats()
    tuned.close()
    assert st.trace_variant < st.trace_variants and all(st.tune_ms[k] > 0 for k in range(st.trace_variants))
    for a, b in zip(ref, outs):
        assert np.array_equal(a.view(np.uint32), b.cpu().numpy().view(np.uint32))
    for k in range(st.trace_variants):
        for per_sm in (0, 2):  # one warp per tile, or a persistent wave of 2 CTAs per SM on a work counter
            srv = fx.server(slots=1, trace_variant=k, blocks_per_sm=per_sm)
            views, outs = fx.make_views(si, vids)
            srv.wait(srv.submit(si, views, []))
            assert srv.stats().trace_variant == k
            srv.close()
            for a, b in zip(ref, outs):
                assert np.array_equal(a.view(np.uint32), b.cpu().numpy().view(np.uint32)), (k, per_sm)


@pytest.mark.gpu
def test_submit_many_shares_one_batch(fx):
    """Requests queued together on distinct scenes run as one batch and give the bytes of separate requests."""
    srv = fx.server(slots=1, max_batch_views=64)
    picks = [(0, [0, 1]), (1, [2]), (2, [0, 3])]
    alone = []
    for si, vids in picks:
        views, outs = fx.make_views(si, vids)
        srv.wait(srv.submit(si, views, []))
        alone.append([o.cpu().numpy() for o in outs])
    keep, reqs = [], []
    for si, vids in picks:
        views, outs = fx.make_views(si, vids)
        keep.append(outs)
        reqs.append((si, views, []))
    res = [srv.wait(t) for t in srv.submit_many(reqs)]
    srv.close()
    assert len({r.batch for r in res}) == 1
    for a, b in zip(alone, keep):
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.cpu().numpy().view(np.uint32))


@pytest.mark.gpu
def test_host_buffer_requests_match_device_requests(fx):
    g = fx.g
    srv = fx.server(slots=2)
    si, vids = 1, [0, 2]
    views, outs = fx.make_views(si, vids)
    srv.wait(srv.submit(si, views, []))
    dev = [o.cpu().numpy() for o in outs]
    hviews, host_out, keep = [], [], []
    for vi in vids:
        V, P, W, H, d, nr, rg = fx.views[(si, vi)]
        hd, hn, hr = d.cpu().numpy(), nr.cpu().numpy(), rg.cpu().numpy()
        ho = np.zeros(2 * W * H * 4, np.float32)
        keep += [hd, hn, hr]
        host_out.append(ho)
        hviews.append(g.make_view(V, P, W, H, hd.ctypes.data, hn.ctypes.data, hr.ctypes.data, ho.ctypes.data))
    srv.wait(srv.submit(si, hviews, [], host_buffers=True))
    srv.close()
    for a, b in zip(dev, host_out):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.gpu
def test_admission_budget_cancel_and_timeout(fx):
    g = fx.g
    # a budget too small for the scene (a 64^3 FP16 chain with resident weights takes ~15 MB) is refused
    srv = g.Server(0, hbm_budget=4 << 20)
    with pytest.raises(g.F184Error) as e:
        sc = fx.scenes[0]
        srv.add_scene(0, fx.desc, sc.tri_xyz, sc.albedo, sc.bounds, sc.light)
    assert e.value.code == g._abi.ERR_BUDGET
    srv.close()
    # a host-buffer request whose staging can never fit is refused at submission
    srv = fx.server(slots=1, hbm_budget=2 << 30)
    big = 1 << 14  # the largest view side: 16384^2 pixels stage ~11 GB of G-buffer and output
    bogus = np.zeros(16, np.float32)
    v = g.make_view(np.eye(4), g.perspective(59.0, 1.0, 0.1, 100.0), big, big, bogus.ctypes.data, bogus.ctypes.data,
                    bogus.ctypes.data, bogus.ctypes.data)
    with pytest.raises(g.F184Error) as e:
        srv.submit(0, [v], [], host_buffers=True)
    assert e.value.code == g._abi.ERR_BUDGET
    # queue several requests on one slot: the last is still pending and can be cancelled
    tickets = []
    keep = []
    for k in range(6):
        views, outs = fx.make_views(k % 3, [0, 1, 2, 3])
        keep.append(outs)
        nt = fx.scenes[k % 3].ntris
        moves = [m for m in fx.requests[k][2] if m[0] + m[1] <= nt]
        tickets.append(srv.submit(k % 3, views, moves))
    # the last request is still pending and can be cancelled; then bounded waits of 1 ms on the requests queued
    # behind the first one (a fresh server's first batch also tunes the kernel variants, so the queue takes many
    # milliseconds): the wait on the last of them must expire, and an expired wait leaves its request to complete
    srv.cancel(tickets[-1])
    expired = []
    for t in reversed(tickets[1:-1]):
        try:
            srv.wait(t, timeout_ms=1)
        except g.F184Error as ex:
            assert ex.code == g._abi.ERR_TIMEOUT
            expired.append(t)
    assert tickets[-2] in expired
    r = srv.wait(tickets[-1])
    assert r.status == g._abi.ERR_CANCELLED
    for t in tickets[:-1]:
        assert srv.wait(t).status == 0
    with pytest.raises(g.F184Error):
        srv.cancel(tickets[0])  # already done
    st = srv.stats()
    assert st.requests_done == 5 and st.requests_cancelled == 1
    srv.close()


@pytest.mark.gpu
def test_injected_update_failure_fails_only_that_request(fx, tmp_path):
    """Host-side fault injection on the real server: one request of a batch fails in its scene update (as if a CUDA
    call had failed, before any of its device work); the others of the batch complete with the bytes they give
    alone, and the server keeps serving.  Every finished request leaves one JSON line in the server's log."""
    g = fx.g
    srv = fx.server(slots=1, max_batch_views=32)
    log = tmp_path / "requests.jsonl"
    srv.set_log(log)
    reqs = [(0, [0, 1], []), (1, [2], []), (2, [0, 3], [])]
    alone = []
    for si, vids, moves in reqs:
        views, outs = fx.make_views(si, vids)
        srv.wait(srv.submit(si, views, moves))
        fx.torch.cuda.synchronize()
        alone.append([o.cpu().numpy().copy() for o in outs])
    made = [fx.make_views(si, vids) for si, vids, _ in reqs]
    t0, bad, t2 = srv.submit_many([(reqs[0][0], made[0][0], []), (reqs[1][0], made[1][0], [], g._abi.REQ_INJECT_FAIL),
                                   (reqs[2][0], made[2][0], [])])
    with pytest.raises(g.F184Error) as e:
        srv.wait(bad)
    assert e.value.code == g._abi.ERR_CUDA
    r0, r2 = srv.wait(t0), srv.wait(t2)
    assert r0.status == 0 and r2.status == 0
    assert r0.batch == r2.batch  # the failed request's batch ran
    fx.torch.cuda.synchronize()
    for k in (0, 2):
        for a, o in zip(alone[k], made[k][1]):
            assert np.array_equal(a.view(np.uint32), o.cpu().numpy().view(np.uint32))
    # the server keeps serving after the failure
    views, outs = fx.make_views(1, [2])
    assert srv.wait(srv.submit(1, views, [])).status == 0
    srv.close()
    import json
    lines = [json.loads(x) for x in open(log)]
    assert len(lines) == 7 and sum(x["status"] == g._abi.ERR_CUDA for x in lines) == 1
