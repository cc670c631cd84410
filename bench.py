"""Benchmark of the voxel cone-tracing GI path on GB300.

One step = one request of the plain per-request path on the large synthetic scene: shadow-map raster +
conservative voxelization with light injection (f184gi_voxelize), the mip chain (f184gi_mip) and the cone trace of
one 1920x1080 view (f184gi_trace).  The metric is cone-traced Mpix/s (pixels traced / time).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--small]

With N > 1 (launched by torch.distributed.run) every rank runs an independent replica of the request on its own
GPU (the path has no data exchange between requests); value = all ranks' pixels / the slowest rank's time.
--impl reference times the CPU restatement of the path (FP32, all host threads) on a bounded sample of the same
workload.  Prints one JSON line on rank 0.
"""
import argparse
import json
import math
import os
import statistics
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cone-traced Mpix/s, p50/p99 latency @<=1e-3 rel err, served vs plain, 1 GB300"
PLAIN_LARGE = dict(name="plain-large", seed=1184, ntris=500000, nobjects=2000, dim=256, levels=8, shadow_res=2048,
                   width=1920, height=1080)
SMALL = dict(name="plain-small-gpu", seed=184, ntris=20000, nobjects=200, dim=64, levels=6, shadow_res=1024,
             width=640, height=360)
E2E_LANES = 1  # compute lanes of the end-to-end measurement (each its own context, grid and stream)


def workload_desc(cfg, storage="f32"):
    return ("%s: %dk-triangle seeded scene (%d objects), %d^3 %s RGBA radiance/opacity grid in 8^3 bricks, "
            "%d-level mip chain, %d^2 shadow map, %dx%d G-buffer, 5 diffuse (60 deg) + 1 specular cone, "
            "max distance = grid diagonal, step = 0.5 x diameter"
            % (cfg["name"], cfg["ntris"] // 1000, cfg["nobjects"], cfg["dim"], "FP16" if storage == "f16" else "FP32",
               cfg["levels"], cfg["shadow_res"], cfg["width"], cfg["height"]))


def bench_config(cfg, storage="f32"):
    """The `config` of both arms (the same keys and values for the same workload)."""
    esz = 8 if storage == "f16" else 16
    chain_mb = sum((cfg["dim"] >> l) ** 3 for l in range(cfg["levels"])) * esz // 2 ** 20
    return {"workload": workload_desc(cfg, storage),
            "l2": "per-step working set > 129 MB L2 (the %d MB grid chain is rewritten and re-read every step)"
                  % chain_mb}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_record(kernel):
    """DRAM bytes per launch of `kernel` (or another figure keyed `kernel`) from the committed ncu summary (None when
    absent)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        t = json.load(f)
    return t.get(kernel)


class ClockSampler:
    """SM clock and clock-event reasons sampled every 10 ms through NVML (read only) during the timed region,
    which begin() and end() bracket."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, device):
        import ctypes as C
        import threading

        self.C, self.samples, self.t0, self.t1 = C, [], None, None
        self.stop_flag = threading.Event()
        self.thread = None
        self.nvml = self.handle = None
        try:
            nvml = C.CDLL("libnvidia-ml.so.1")
            if nvml.nvmlInit_v2() != 0:
                return
            h = C.c_void_p()
            bus = self._bus_id(device)
            ok = bus is not None and nvml.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), C.byref(h)) == 0
            if not ok and nvml.nvmlDeviceGetHandleByIndex_v2(C.c_uint(device.index or 0), C.byref(h)) != 0:
                return
            self.nvml, self.handle = nvml, h
            self.reasons_fn = getattr(nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nvml.nvmlDeviceGetCurrentClocksThrottleReasons
        except (OSError, AttributeError):
            self.nvml = None

    @staticmethod
    def _bus_id(device):
        import torch

        p = torch.cuda.get_device_properties(device)
        if not hasattr(p, "pci_bus_id"):
            return None
        return "%08x:%02x:%02x.0" % (getattr(p, "pci_domain_id", 0), p.pci_bus_id, getattr(p, "pci_device_id", 0))

    def _read(self):
        C = self.C
        clk, mx, r = C.c_uint(0), C.c_uint(0), C.c_ulonglong(0)
        if self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, C.byref(clk)) != 0:
            return None
        self.nvml.nvmlDeviceGetMaxClockInfo(self.handle, 1, C.byref(mx))
        self.reasons_fn(self.handle, C.byref(r))
        return time.time(), clk.value, mx.value, r.value

    def _loop(self):
        while not self.stop_flag.is_set():
            s = self._read()
            if s:
                self.samples.append(s)
            time.sleep(0.01)

    def start(self):
        if self.nvml is None:
            return
        import threading

        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def stop(self):
        if self.thread is None:
            return None
        self.stop_flag.set()
        self.thread.join()
        t0, t1 = self.t0 or 0.0, self.t1 or time.time()
        win = [s for s in self.samples if t0 <= s[0] <= t1]
        if not win:  # a region shorter than the sampling period: the samples nearest to it
            win = sorted(self.samples, key=lambda s: abs(s[0] - 0.5 * (t0 + t1)))[:2]
        if not win:
            return None
        reasons = sorted({n for s in win for bit, n in self.REASONS.items() if s[3] & bit})
        return {"sm_mhz": statistics.median([s[1] for s in win]), "sm_max_mhz": max(s[2] for s in win),
                "reasons": reasons, "samples": len(win), "source": "NVML, every 10 ms over the timed region"}


def slowest_rank_ms(local_ms, device=None):
    """The largest per-rank time (replicas report the slowest rank; a no-op for one process)."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(local_ms)
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_mpix(units_per_rank, slowest_ms, world):
    """Whole-job throughput of `world` replicas that each processed units_per_rank pixels in at most slowest_ms."""
    return world * units_per_rank / (slowest_ms * 1e-3) / 1e6


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- CPU restatement (baseline / reference arm)

def cpu_request(cfg, row_stride, scene=None, f64_check=None):
    """Time the FP32 CPU restatement of one request on a row sample; returns (seconds per full request, info).
    The scene and cameras come from the host-only build of the seeded generator (the CUDA library is not loaded)."""
    import numpy as np

    import oracle as o
    from oracle import scene_host

    sc = scene or scene_host.HostScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    dim, levels, res, W, H = cfg["dim"], cfg["levels"], cfg["shadow_res"], cfg["width"], cfg["height"]
    ld = np.array(sc.light.direction, np.float32)
    b = sc.bounds
    light = o.make_light(list(sc.light.luminance), list(sc.light.direction))
    t0 = time.perf_counter()
    fo = o.grid_frame(o.make_bounds((b.min.x, b.min.y, b.min.z), (b.max.x, b.max.y, b.max.z)), dim, ld)
    sd = o.shadow_depth(o.raster(o.frame_matrix(fo), res, res, sc.tri_xyz))
    l0, _ = o.voxelize(fo, dim, res, sc.tri_xyz, sc.albedo, light, sd, f64=False)
    chain, _ = o.mip(l0, levels, f64=False)
    t1 = time.perf_counter()
    gb = cpu_gbuffer(sc, cfg)
    V, P, dep, nrm, rgh = gb
    rows = list(range(0, H, row_stride))
    t2 = time.perf_counter()
    outs = {}
    if row_stride == 1:  # the whole image in one call (all threads over all pixels)
        img = o.trace(fo, dim, levels, chain, V, P, W, H, dep, nrm, rgh, f64=False)
        outs = {r: img[:, r] for r in rows}
    else:
        for r in rows:
            outs[r] = o.trace(fo, dim, levels, chain, V, P, W, H, dep, nrm, rgh, rows=(r, r + 1), f64=False)[:, r]
    t3 = time.perf_counter()
    per_request = (t1 - t0) + (t3 - t2) * H / len(rows)
    info = {"voxelize_mip_s": t1 - t0, "trace_rows": len(rows), "trace_s": t3 - t2}
    return per_request, info, (sc, fo, chain, gb, outs)


def cpu_gbuffer(sc, cfg):
    import numpy as np

    import oracle as o
    from oracle import scene_host

    W, H = cfg["width"], cfg["height"]
    V = scene_host.look_at(sc.eye, sc.target)
    P = scene_host.perspective(59.0, W / H, 0.1, 100.0)
    keys = o.raster(P.astype(np.float64) @ V.astype(np.float64), W, H, sc.tri_xyz)
    dep, nrm, rgh, _ = o.gbuffer_resolve(keys, sc.tri_xyz, sc.roughness, V)
    return V, P, dep, nrm, rgh


def run_reference(args, cfg):
    """--impl reference: the CPU restatement, all host threads, each step a bounded row sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    from oracle import build as ob
    from oracle import scene_host

    ob.build_oracle()
    sc = scene_host.HostScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    for _ in range(min(args.warmup, 1)):
        cpu_request(cfg, 64, scene=sc)
    # each step is the whole request (voxelization, mips, every row of the trace) while K of them fit in about
    # two minutes; beyond that a step traces every stride-th row and scales the trace time to the full image
    t_full, info, _ = cpu_request(cfg, 1, scene=sc)
    budget = max(0.05, 120.0 / max(1, args.steps))
    stride = 1
    if t_full > budget:
        stride = min(cfg["height"], math.ceil(info["trace_s"] / max(budget - info["voxelize_mip_s"], 0.01)))
    times = [t_full]
    for _ in range(args.steps - 1):
        t, info, _ = cpu_request(cfg, stride, scene=sc)
        times.append(t)
    t = statistics.mean(times)
    mpix = cfg["width"] * cfg["height"] / t / 1e6
    cores = os.cpu_count() or 1
    sample = ("per step: the whole request on the CPU: shadow raster + voxelization + mip chain of the scene and the "
              "cone trace of %s" % ("all %d rows" % cfg["height"] if stride == 1 else
                                    "every %d-th row (the first step: all rows), scaled to the image" % stride))
    line = {"metric": METRIC, "impl": "reference", "value": round(mpix, 4), "unit": "Mpix/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(cfg),
            "implementation": "CPU restatement of the path (oracle.cpp) in FP32, std::thread over all host cores; "
                              "scenes and cameras from the host-only build of the seeded generator",
            "cpu_baseline": {"value": round(mpix, 4), "unit": "Mpix/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(mpix, 4), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


# ---------------------------------------------------------------- GPU arm

def issue_roofline(warp_inst, ms, dev, clk):
    """The trace kernel against the SM issue peak: warp instructions per launch (the committed ncu capture of the
    same kernel on the same view) / its CUDA-event time, over SMs x 4 schedulers x the SM clock sampled during the
    timed region (one warp instruction per scheduler per cycle)."""
    if not warp_inst or not ms:
        return None
    import torch

    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6
    achieved = warp_inst / (ms * 1e-3)
    return {"bound": "issue", "achieved": round(achieved / 1e9, 2), "peak": round(peak / 1e9, 2),
            "unit": "G warp instructions/s", "frac": round(achieved / peak, 4), "warp_instructions": int(warp_inst),
            "source": "warp instructions from profiles/trace_kernel_plain-large.md (ncu, FP32 chain); peak = %d SMs x "
                      "4 schedulers x %.0f MHz" % (sms, mhz)}


def l2_copy_gbs(dev, stream, mib=40, reps=100):
    """Read + write GB/s of a device copy whose source and destination (2 x mib MiB) stay in L2."""
    import torch

    a = torch.empty(mib << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    a.fill_(1)
    for _ in range(10):
        b.copy_(a)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.copy_(a)
    e1.record(stream)
    e1.synchronize()
    return 2.0 * a.numel() * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9


def run_gpu(args, cfg):
    import numpy as np
    import torch

    import final184_gb300 as g

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sc = g.SyntheticScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    gi = g.VoxelGI(local)
    dim, levels, res, W, H = cfg["dim"], cfg["levels"], cfg["shadow_res"], cfg["width"], cfg["height"]
    fmt = g.FMT_F16 if args.storage == "f16" else g.FMT_F32
    grid = gi.create_grid(dim, levels, fmt, 0, res)
    npix = W * H
    # host inputs (pinned) and device copies
    tri_h = torch.from_numpy(sc.tri_xyz).pin_memory()
    alb_h = torch.from_numpy(sc.albedo.view(np.int32)).pin_memory()
    tri = tri_h.to(dev)
    alb = alb_h.to(dev)
    rough = torch.from_numpy(sc.roughness).to(dev)
    V = g.look_at(sc.eye, sc.target)
    P = g.perspective(59.0, W / H, 0.1, 100.0)
    depth = torch.empty(npix, dtype=torch.float32, device=dev)
    normal = torch.empty(npix, dtype=torch.int32, device=dev)
    rgh = torch.empty(npix, dtype=torch.int16, device=dev)
    out = torch.empty(2 * npix * 4, dtype=torch.float32, device=dev)
    view = g.make_view(V, P, W, H, depth.data_ptr(), normal.data_ptr(), rgh.data_ptr(), out.data_ptr())
    # the G-buffer is the trace's input (the reference's G-buffer pass); rasterized once, outside the timing
    gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view, stream=stream)
    gi.sync(stream)
    gbuf_h = [depth.cpu().pin_memory(), normal.cpu().pin_memory(), rgh.cpu().pin_memory()]
    out_h = torch.empty(out.numel(), dtype=torch.float32).pin_memory()
    light = sc.light

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, light, bounds=sc.bounds, stream=stream)
        if ev is not None:
            ev[1].record(stream)
        gi.mip(grid, stream=stream)
        if ev is not None:
            ev[2].record(stream)
        gi.trace(grid, [view], stream=stream)
        if ev is not None:
            ev[3].record(stream)

    for _ in range(args.warmup):
        step()
    gi.sync(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # ---- device-resident timing ----
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    clocks = ClockSampler(dev)
    clocks.start()
    launches0 = g.load().f184gi_kernel_launches()
    barrier()
    clocks.begin()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    barrier()
    clocks.end()
    launches = g.load().f184gi_kernel_launches() - launches0
    clk = clocks.stop()
    gi.sync(stream)
    total_ms = slowest_rank_ms(t_start.elapsed_time(t_end), dev)
    ms_per_step = total_ms / args.steps
    step_ms = [evs[k][0].elapsed_time(evs[k][3]) for k in range(args.steps)]
    stage = {"voxelize": [e[0].elapsed_time(e[1]) for e in evs], "mip": [e[1].elapsed_time(e[2]) for e in evs],
             "trace": [e[2].elapsed_time(e[3]) for e in evs]}
    value = replica_mpix(npix, ms_per_step, world)
    ref_img = out.cpu().numpy().view(np.uint32).copy()  # the device-timed loop's image

    # ---- end to end through the API with host buffers ----
    # E2E_LANES compute lanes (each its own context, grid and stream) take the requests in turn; the copies run on
    # one copy-in and one copy-out stream, in request order, into and out of 2 x E2E_LANES sets of device buffers,
    # so a request's inputs arrive and its image leaves while other requests compute.  Every step still copies its
    # inputs in from pinned host memory and its traced image out.  Measured per plain-large request: one lane
    # 2.253 ms (two runs), two lanes 2.251-2.277, three 2.271-2.308 (requests computing at the same time share the
    # SMs badly: the bricks' shared memory takes L1 from a concurrent trace); lanes that carried their own copies
    # in order on their streams 2.38 ms with two (both lanes copying at once while the GPU idles) and 2.20-2.31 ms
    # with three.
    h2d = tri_h.numel() * 4 + alb_h.numel() * 4 + sum(x.numel() * x.element_size() for x in gbuf_h)
    d2h = out.numel() * 4
    lanes = [dict(gi=gi, grid=grid, stream=stream)]
    for _ in range(E2E_LANES - 1):
        gl = g.VoxelGI(local)
        lanes.append(dict(gi=gl, grid=gl.create_grid(dim, levels, fmt, 0, res), stream=torch.cuda.Stream(dev)))
    sets = [dict(tri=tri, alb=alb, gbuf=[depth, normal, rgh], out=out, out_h=out_h, view=view)]
    for _ in range(2 * E2E_LANES - 1):
        dl = [torch.empty_like(depth), torch.empty_like(normal), torch.empty_like(rgh)]
        ol = torch.empty_like(out)
        sets.append(dict(tri=torch.empty_like(tri), alb=torch.empty_like(alb), gbuf=dl, out=ol,
                         out_h=torch.empty_like(out_h).pin_memory(),
                         view=g.make_view(V, P, W, H, dl[0].data_ptr(), dl[1].data_ptr(), dl[2].data_ptr(),
                                          ol.data_ptr())))
    for S in sets:
        S.update(in_ready=torch.cuda.Event(), in_free=torch.cuda.Event(), out_ready=torch.cuda.Event(),
                 out_free=torch.cuda.Event())
    cin, cout = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def e2e_step(k):
        S, L = sets[k % len(sets)], lanes[k % len(lanes)]
        with torch.cuda.stream(cin):  # inputs in, once the request that last used this set has read them
            cin.wait_event(S["in_free"])
            S["tri"].copy_(tri_h, non_blocking=True)
            S["alb"].copy_(alb_h, non_blocking=True)
            for d_, h_ in zip(S["gbuf"], gbuf_h):
                d_.copy_(h_, non_blocking=True)
            S["in_ready"].record(cin)
        ls = L["stream"]
        ls.wait_event(S["in_ready"])
        ls.wait_event(S["out_free"])  # its image buffer copied out
        L["gi"].voxelize(L["grid"], S["tri"].data_ptr(), S["alb"].data_ptr(), sc.ntris, light, bounds=sc.bounds,
                         stream=ls)
        L["gi"].mip(L["grid"], stream=ls)
        L["gi"].trace(L["grid"], [S["view"]], stream=ls)
        S["in_free"].record(ls)
        S["out_ready"].record(ls)
        with torch.cuda.stream(cout):
            cout.wait_event(S["out_ready"])
            S["out_h"].copy_(S["out"], non_blocking=True)
            S["out_free"].record(cout)

    for k in range(len(sets)):  # warm every lane and buffer set
        e2e_step(k)
    torch.cuda.synchronize(dev)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for st in [cin, cout] + [L["stream"] for L in lanes[1:]]:
        st.wait_event(e0)
    for k in range(args.steps):
        e2e_step(k)
    for st in [cout] + [L["stream"] for L in lanes[1:]]:
        done = torch.cuda.Event()
        done.record(st)
        stream.wait_event(done)
    e1.record(stream)
    barrier()
    e2e_ms = slowest_rank_ms(e0.elapsed_time(e1) / args.steps, dev)
    e2e_value = replica_mpix(npix, e2e_ms, world)
    # every request traces the same inputs: the images copied out to the host equal the device-timed loop's
    torch.cuda.synchronize(dev)
    e2e_same = all(bool(np.array_equal(S["out_h"].numpy().view(np.uint32), ref_img)) for S in sets)

    # ---- roofline of the dominant kernel (HBM: nothing here is a dense contraction) ----
    # trace_kernel is the largest single kernel of a request (launch-list share ~42%); its stage is one launch
    means = {k: statistics.mean(v) for k, v in stage.items()}
    top = "trace"
    esz = 8 if args.storage == "f16" else 16
    chain_bytes = sum((dim >> l) ** 3 for l in range(levels)) * esz
    l0_bytes = dim ** 3 * esz
    alg = {
        # triangles + albedo read, L0 written once, shadow map written and read once (4 B/texel)
        "voxelize": sc.ntris * 40 + l0_bytes + 2 * 4 * res * res,
        # L0 read once, levels 1.. written once
        "mip": chain_bytes,
        # G-buffer 10 B + 2 x RGBA FP32 out per pixel; the chain counted once per launch (upper bound of touched)
        "trace": npix * (10 + 32) + chain_bytes,
    }
    peak, peak_kind = peaks()
    achieved = alg[top] / (means[top] * 1e-3) / 1e9
    # secondary figure: the voxel bytes the trace samples (8 taps x esz B per level sample), counted by the
    # instrumented kernel on the same view after the timed region, against an L2-resident copy measured here
    n_steps, n_samples = gi.trace_count(grid, [view], stream=stream)
    sampled = n_samples * 8 * esz
    l2_gbs = l2_copy_gbs(dev, stream)
    kernel_names = {"voxelize": "vox_bricks", "mip": "mip_pass", "trace": "trace_kernel"}
    tr = traffic_record(kernel_names[top] + ("_f16" if args.storage == "f16" else ""))
    tr_inst = traffic_record(kernel_names[top] + ("_f16" if args.storage == "f16" else "") + "_warp_instructions")
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(cfg, args.storage),
        "form": "plain per-request %s GPU path" % ("FP32" if args.storage == "f32" else "FP16-storage"),
        "parallelism": "replicas" if world > 1 else "single GPU",
        "latency_ms": {"p50": round(statistics.median(step_ms), 4),
                       "p99": round(sorted(step_ms)[min(len(step_ms) - 1, int(0.99 * len(step_ms)))], 4)},
        "stages_ms": {k: round(v, 4) for k, v in means.items()},
        "roofline": {"bound": "hbm", "kernel": kernel_names[top], "achieved": round(achieved, 2), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "algorithmic_bytes": alg[top],
                     "traffic": (tr * 1.0 if isinstance(tr, (int, float)) else None),
                     "note": "far below the HBM roof: the trace is bound by instruction issue and the L1 load pipe "
                             "together (ncu: ~69% issue-active, load-pipe wavefronts ~75%, L1 hit ~96%, DRAM ~0.4% of "
                             "peak; see `issue`); algorithmic bytes = G-buffer 10 B + output "
                             "32 B per pixel + the whole chain once (upper bound of the touched part)",
                     "issue": issue_roofline(tr_inst, means[top], dev, clk),
                     "sampled": {"bytes": int(sampled), "achieved": round(sampled / (means[top] * 1e-3) / 1e9, 1),
                                 "unit": "GB/s", "l2_copy_gbs": round(l2_gbs, 1),
                                 "frac_of_l2_copy": round(sampled / (means[top] * 1e-3) / 1e9 / l2_gbs, 3),
                                 "steps_per_pixel": round(n_steps / max(1, npix), 2),
                                 "level_samples_per_pixel": round(n_samples / max(1, npix), 2),
                                 "note": "secondary figure, not the roofline: voxel bytes sampled by the cones "
                                         "(level samples x 8 taps x %d B, counted by the instrumented kernel) per "
                                         "trace launch time; most are L1 hits, so it may exceed the L2 figure, "
                                         "a torch copy of 2 x 40 MiB held in L2" % esz}},
        "e2e": {"value": round(e2e_value, 4), "unit": "Mpix/s", "h2d_bytes_per_step": int(h2d),
                "images_equal_device_loop": e2e_same,
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 4),
                "note": "through the API from pinned host buffers; %d compute lanes (context, grid, stream) take the "
                        "requests in turn, their copies on a copy-in and a copy-out stream into and out of %d device "
                        "buffer sets, so a request's copies overlap other requests' kernels" % (len(lanes), len(sets))},
        "gpu_launches": int(launches),
        "clocks": clk,
        # the traced image is lit (a black image would trace trivially short cones)
        "image": {"mean_diffuse_rgb": round(float(out.view(2, -1, 4)[0, :, :3].mean()), 6),
                  "mean_specular_rgb": round(float(out.view(2, -1, 4)[1, :, :3].mean()), 6)},
    }
    if world > 1:
        torch.distributed.barrier()
    for L in lanes[1:]:
        L["gi"].close()
    gi.close()
    return line, sc


SERVED = dict(scenes=[(128, 7, 100000, 400), (128, 7, 200000, 800), (256, 8, 300000, 1200), (256, 8, 500000, 2000)],
              requests=120, rate=200.0, max_moved=0.05, views=(1, 16), sizes=((512, 512), (1920, 1080)),
              shadow_res=2048, seed=4242, budget=120 << 30)


def run_served(args, cfg=SERVED):
    """Served form vs the plain per-request path on the same seeded request stream (one GPU).

    Every view of every request has its own seeded camera (no two views share a G-buffer).  Both arms see the same
    arrival times: the served arm submits each request when it arrives and the server batches what is pending; the
    plain arm takes the requests one at a time in arrival order (FIFO), a request starting when it has arrived and
    the previous one is done.  A request's latency is its completion time minus its arrival time in both arms."""
    import threading

    import numpy as np
    import torch

    import final184_gb300 as g

    rng = np.random.default_rng(cfg["seed"])
    dev = torch.device("cuda", 0)
    scenes = []
    gi = g.VoxelGI(0)
    for k, (dim, levels, ntris, nobj) in enumerate(cfg["scenes"]):
        sc = g.SyntheticScene(cfg["seed"] + 100 * k, ntris, nobj)
        scenes.append((sc, dim, levels))
    # the request stream: Poisson arrivals, 0..5% of a scene's objects moved, 1..16 views with cameras of their own
    reqs, t = [], 0.0
    for i in range(cfg["requests"]):
        t += rng.exponential(1.0 / cfg["rate"])
        si = int(rng.integers(0, len(scenes)))
        sc = scenes[si][0]
        nmov = int(rng.integers(0, int(cfg["max_moved"] * (sc.nobjects - 1)) + 1))
        moves = []
        for o in rng.choice(np.arange(1, sc.nobjects), nmov, replace=False):
            moves.append((int(sc.object_first[o]), int(sc.object_count[o]),
                          [float(x) for x in rng.uniform(-0.2, 0.2, 3).astype(np.float32)]))
        nv = int(rng.integers(cfg["views"][0], cfg["views"][1] + 1))
        cams = []
        for j in range(nv):
            (w0, h0), (w1, h1) = cfg["sizes"]
            u = rng.uniform(0, 1)
            cams.append((int(w0 + u * (w1 - w0)) // 8 * 8, int(h0 + u * (h1 - h0)) // 8 * 8))
        reqs.append((t, si, moves, cams))
    # G-buffers (the trace's inputs) of every view, rasterized from the scenes' initial geometry outside the timing
    gbufs = []
    for i, (_, si, _, cams) in enumerate(reqs):
        sc = scenes[si][0]
        tri = torch.from_numpy(sc.tri_xyz).to(dev)
        rough = torch.from_numpy(sc.roughness).to(dev)
        row = []
        for j, (W, H) in enumerate(cams):
            eye, tgt = sc.camera(j, seed=cfg["seed"] * 1000 + i)
            V, P = g.look_at(eye, tgt), g.perspective(59.0, W / H, 0.1, 100.0)
            n = W * H
            bufs = (torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.int32, device=dev),
                    torch.empty(n, dtype=torch.int16, device=dev))
            gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, g.make_view(V, P, W, H, bufs[0].data_ptr(),
                                                                                  bufs[1].data_ptr(), bufs[2].data_ptr(), 0))
            row.append((V, P, W, H, bufs))
        gbufs.append(row)
        del tri, rough
    gi.sync()
    pixels = sum(W * H for _, _, _, cams in reqs for W, H in cams)
    max_px = max(W * H for _, _, _, cams in reqs for W, H in cams)
    outs = [torch.empty(2 * max_px * 4, dtype=torch.float16, device=dev) for _ in range(16)]

    def views_for(i, fmt):
        vs = []
        for j, (V, P, W, H, b) in enumerate(gbufs[i]):
            vs.append(g.make_view(V, P, W, H, b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(), outs[j].data_ptr(),
                                  fmt))
        return vs

    def pct(lat, q):
        return round(lat[min(len(lat) - 1, int(q * len(lat)))], 2)

    def served_arm(time_scale, fmt=g.FMT_F16):
        """`fmt` grids (FP16 by default) with resident weights, continuous batching, arrivals in real time at the
        stream's arrival times x time_scale; returns (wall seconds, sorted request latencies in ms, views per
        batch)."""
        srv = g.Server(0, slots=2, max_batch_views=64, hbm_budget=cfg["budget"])
        for k, (sc, dim, levels) in enumerate(scenes):
            srv.add_scene(k, g.GridDesc(dim, levels, fmt, 0, cfg["shadow_res"], 0), sc.tri_xyz, sc.albedo,
                          sc.bounds, sc.light)
        # warm-up, outside the timing: one request per scene (the first batch tunes the trace kernel variant;
        # graphs, staging and scratch are set up)
        warm = []
        for k in range(len(scenes)):
            i = next(i for i, r in enumerate(reqs) if r[1] == k)
            warm.append(srv.submit(k, views_for(i, fmt), []))
        for tk in warm:
            srv.wait(tk)
        tickets = [None] * len(reqs)

        def submitter():
            t0 = time.perf_counter()
            for i, (ta, si, moves, _) in enumerate(reqs):
                d = ta * time_scale - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                tickets[i] = srv.submit(si, views_for(i, fmt), moves)

        w0 = time.perf_counter()
        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        results = [srv.wait(tk) for tk in tickets]
        wall = time.perf_counter() - w0
        srv.close()
        per_batch = {}  # batches of the timed stream -> their views
        for r, (_, _, _, cams) in zip(results, reqs):
            per_batch[r.batch] = per_batch.get(r.batch, 0) + len(cams)
        return wall, sorted(r.latency_ms for r in results), per_batch

    # ---- served: the stream at its rate, then at a third of it (a load the server sustains without a queue) ----
    served_s, served_lat, batch_views = served_arm(1.0)
    light_s, light_lat, light_batches = served_arm(3.0)

    def plain_arm(fmt):
        """The same stream, one request at a time in arrival order (FIFO) at the same arrival times: full
        voxelization, mips and one trace launch per view, `fmt` grids and output; returns (Mpix/s, sorted request
        latencies in ms from arrival to completion, wall seconds)."""
        lat = []
        geo = [sc.tri_xyz.copy() for sc, _, _ in scenes]
        grids = [gi.create_grid(dim, levels, fmt, 0, cfg["shadow_res"]) for _, dim, levels in scenes]
        dtri = [torch.from_numpy(x).to(dev) for x in geo]
        dalb = [torch.from_numpy(sc.albedo.view(np.int32)).to(dev) for sc, _, _ in scenes]
        odt = torch.float32 if fmt == g.FMT_F32 else torch.float16
        outs[:] = [torch.empty(2 * max_px * 4, dtype=odt, device=dev) for _ in range(16)]
        for si, (sc, _, _) in enumerate(scenes):  # warm-up, outside the timing: scratch and first launches
            i = next(i for i, r in enumerate(reqs) if r[1] == si)
            gi.voxelize(grids[si], dtri[si].data_ptr(), dalb[si].data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
            gi.mip(grids[si])
            gi.trace(grids[si], views_for(i, fmt)[:1])
        gi.sync()
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        for i, (ta, si, moves, _) in enumerate(reqs):
            d = ta - (time.perf_counter() - p0)
            if d > 0:
                time.sleep(d)
            sc = scenes[si][0]
            for f, c, off in moves:  # the caller moves its geometry and re-uploads it
                seg = geo[si][f * 9:(f + c) * 9].reshape(-1, 3)
                seg += np.asarray(off, dtype=np.float32)
            dtri[si].copy_(torch.from_numpy(geo[si]))
            gi.voxelize(grids[si], dtri[si].data_ptr(), dalb[si].data_ptr(), sc.ntris, sc.light, bounds=sc.bounds)
            gi.mip(grids[si])
            for v in views_for(i, fmt):
                gi.trace(grids[si], [v])
            gi.sync()
            lat.append((time.perf_counter() - p0 - ta) * 1e3)
        wall = time.perf_counter() - p0
        for gr in grids:
            gi.destroy_grid(gr)
        return pixels / wall / 1e6, sorted(lat), wall

    # ---- plain: FP32 grids (the per-request path the served form is held against), then FP16 grids ----
    plain_mpix, plain_lat, plain_s = plain_arm(g.FMT_F32)
    # the served form on the plain path's storage (FP32 grids and images): its serving gain at equal storage
    s32_s, s32_lat, s32_batches = served_arm(1.0, g.FMT_F32)
    p16_mpix, p16_lat, p16_s = plain_arm(g.FMT_F16)
    gi.close()
    served_mpix = pixels / served_s / 1e6
    return {
        "workload": "%d requests, Poisson arrivals at %.0f req/s, 0-5%% of a scene's objects moved, 1-16 views of "
                    "512x512..1920x1080, each view with its own seeded camera, on resident grids %s, %.0f GB admission "
                    "budget; both arms see the same arrival times and are warmed up first (the served form's first "
                    "batch tunes its kernel variant)"
                    % (len(reqs), cfg["rate"], "/".join("%d^3:%dk" % (d, n // 1000) for d, _, n, _ in cfg["scenes"]),
                       cfg["budget"] / 2 ** 30),
        "pixels": int(pixels),
        "served": {"value": round(served_mpix, 2), "unit": "Mpix/s", "p50_ms": pct(served_lat, 0.5),
                   "p99_ms": pct(served_lat, 0.99), "batches": len(batch_views),
                   "mean_batch_views": round(sum(batch_views.values()) / max(1, len(batch_views)), 2),
                   "wall_s": round(served_s, 3),
                   "storage": "fp16, resident weights + dirty-brick re-voxelization"},
        "plain": {"value": round(plain_mpix, 2), "unit": "Mpix/s", "p50_ms": pct(plain_lat, 0.5),
                  "p99_ms": pct(plain_lat, 0.99), "wall_s": round(plain_s, 3),
                  "storage": "fp32, full voxelization per request, one launch per view, FIFO at the same arrivals"},
        "plain_fp16": {"value": round(p16_mpix, 2), "unit": "Mpix/s", "p50_ms": pct(p16_lat, 0.5),
                       "p99_ms": pct(p16_lat, 0.99), "wall_s": round(p16_s, 3),
                       "storage": "fp16, full voxelization per request, one launch per view, FIFO at the same arrivals "
                                  "(the served form's storage without its serving)"},
        "served_sustainable": {
            "rate_req_s": round(cfg["rate"] / 3.0, 1), "value": round(pixels / light_s / 1e6, 2), "unit": "Mpix/s",
            "p50_ms": pct(light_lat, 0.5), "p99_ms": pct(light_lat, 0.99), "batches": len(light_batches),
            "note": "the same requests arriving at a third of the rate: throughput is then the offered load, and the "
                    "latency is the service time without the queue the full-rate stream builds"},
        "served_fp32": {"value": round(pixels / s32_s / 1e6, 2), "unit": "Mpix/s", "p50_ms": pct(s32_lat, 0.5),
                        "p99_ms": pct(s32_lat, 0.99), "batches": len(s32_batches), "wall_s": round(s32_s, 3),
                        "storage": "fp32 (the plain path's), resident weights + dirty-brick re-voxelization; not the "
                                   "north star's FP16 form: its serving gain at equal storage"},
        "served_over_plain": round(served_mpix / plain_mpix, 3),
        "served_over_plain_fp16": round(served_mpix / p16_mpix, 3),
        "served_fp32_over_plain": round(pixels / s32_s / 1e6 / plain_mpix, 3),
    }


PRECISION = dict(name="precision", seed=2184, ntris=2000000, nobjects=8000, dim=512, levels=9, shadow_res=4096,
                 width=3840, height=2160)
BATCHED = dict(seed=3184, scenes=64, dims=(64, 128, 256), tris=(10000, 1000000), views=(1, 8),
               sizes=((256, 256), (1920, 1080)))


def run_precision(args, cfg=PRECISION):
    """Precision form: 512^3 FP16 chain with six-direction anisotropic mips (9 levels), 2M triangles, 3840x2160,
    FP32 cone accumulation (its error against the FP64 oracle is a GPU test)."""
    import numpy as np
    import torch

    import final184_gb300 as g

    dev = torch.device("cuda", 0)
    sc = g.SyntheticScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    gi = g.VoxelGI(0)
    grid = gi.create_grid(cfg["dim"], cfg["levels"], g.FMT_F16, 1, cfg["shadow_res"])
    tri = torch.from_numpy(sc.tri_xyz).to(dev)
    alb = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    rough = torch.from_numpy(sc.roughness).to(dev)
    W, H = cfg["width"], cfg["height"]
    npix = W * H
    V, P = g.look_at(sc.eye, sc.target), g.perspective(59.0, W / H, 0.1, 100.0)
    depth = torch.empty(npix, dtype=torch.float32, device=dev)
    normal = torch.empty(npix, dtype=torch.int32, device=dev)
    rgh = torch.empty(npix, dtype=torch.int16, device=dev)
    out = torch.empty(2 * npix * 4, dtype=torch.float32, device=dev)
    view = g.make_view(V, P, W, H, depth.data_ptr(), normal.data_ptr(), rgh.data_ptr(), out.data_ptr())
    stream = torch.cuda.Stream(dev)
    gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view, stream=stream.cuda_stream)
    gi.sync(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stages = {"voxelize": [], "mip": [], "trace": []}
    steps = max(2, min(args.steps, 5))
    for k in range(2 + steps):
        ev[0].record(stream)
        gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds,
                    stream=stream.cuda_stream)
        ev[1].record(stream)
        gi.mip(grid, stream=stream.cuda_stream)
        ev[2].record(stream)
        gi.trace(grid, [view], stream=stream.cuda_stream)
        ev[3].record(stream)
        gi.sync(stream.cuda_stream)
        if k >= 2:
            stages["voxelize"].append(ev[0].elapsed_time(ev[1]))
            stages["mip"].append(ev[1].elapsed_time(ev[2]))
            stages["trace"].append(ev[2].elapsed_time(ev[3]))
    ms = {k: statistics.mean(v) for k, v in stages.items()}
    step_ms = sum(ms.values())
    res = {"workload": "%dk-triangle seeded scene (%d objects), %d^3 FP16 RGBA chain in 8^3 Morton bricks with "
                       "6-direction anisotropic mips (%d levels), %d^2 shadow map, %dx%d G-buffer, FP32 cone "
                       "accumulation" % (cfg["ntris"] // 1000, cfg["nobjects"], cfg["dim"], cfg["levels"],
                                         cfg["shadow_res"], W, H),
           "value": round(npix / (step_ms * 1e-3) / 1e6, 2), "unit": "Mpix/s", "steps": steps,
           "ms_per_step": round(step_ms, 3), "stages_ms": {k: round(v, 3) for k, v in ms.items()},
           "device_bytes": int(gi.memory_used()),
           "error_vs_fp64": "gated by tests/test_precision_form.py (every 64th row against the FP64 oracle)",
           "image": {"mean_diffuse_rgb": round(float(out.view(2, -1, 4)[0, :, :3].mean()), 6),
                     "mean_specular_rgb": round(float(out.view(2, -1, 4)[1, :, :3].mean()), 6)}}
    gi.close()
    return res


def run_march(args, cfg=PLAIN_LARGE, dim=128):
    """Reference-faithful mode: the reference's 565 volume (dim^3, the reference's 128^3) and its 4-ray march with
    a second bounce over the plain-large view; bit-identical to the FP32 restatement (tests)."""
    import numpy as np
    import torch

    import final184_gb300 as g

    dev = torch.device("cuda", 0)
    sc = g.SyntheticScene(cfg["seed"], cfg["ntris"], cfg["nobjects"])
    gi = g.VoxelGI(0)
    grid = gi.create_grid(dim, 1, g.FMT_RG16, 0, cfg["shadow_res"])
    tri = torch.from_numpy(sc.tri_xyz).to(dev)
    alb = torch.from_numpy(sc.albedo.view(np.int32)).to(dev)
    rough = torch.from_numpy(sc.roughness).to(dev)
    W, H = cfg["width"], cfg["height"]
    npix = W * H
    V, P = g.look_at(sc.eye, sc.target), g.perspective(59.0, W / H, 0.1, 100.0)
    depth = torch.empty(npix, dtype=torch.float32, device=dev)
    normal = torch.empty(npix, dtype=torch.int32, device=dev)
    rgh = torch.empty(npix, dtype=torch.int16, device=dev)
    out = torch.empty(npix * 4, dtype=torch.float32, device=dev)
    view = g.make_view(V, P, W, H, depth.data_ptr(), normal.data_ptr(), rgh.data_ptr(), out.data_ptr())
    stream = torch.cuda.Stream(dev)
    s = stream.cuda_stream
    gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view, stream=s)
    gi.sync(s)
    blurred = torch.empty_like(out)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    vox, mar, blr = [], [], []
    for k in range(3 + max(3, min(args.steps, 10))):
        ev[0].record(stream)
        gi.voxelize(grid, tri.data_ptr(), alb.data_ptr(), sc.ntris, sc.light, bounds=sc.bounds, stream=s)
        ev[1].record(stream)
        gi.march(grid, [view], stream=s)
        ev[2].record(stream)
        gi.blur(out.data_ptr(), depth.data_ptr(), W, H, blurred.data_ptr(), stream=s)  # blurX + blurY
        ev[3].record(stream)
        gi.sync(s)
        if k >= 3:
            vox.append(ev[0].elapsed_time(ev[1]))
            mar.append(ev[1].elapsed_time(ev[2]))
            blr.append(ev[2].elapsed_time(ev[3]))
    img = out.view(-1, 4)[:, :3]
    res = {"workload": "the reference's %d^3 RGB565|normal565 volume (dominant-axis raster of %dk triangles, highest "
                       "triangle wins) and its 4-ray march with second bounce, 60 x 0.2-unit steps, shadow-mapped sun "
                       "and sky, then the two-pass depth-aware blur, over the %dx%d plain-large view" % (dim, cfg["ntris"] // 1000, W, H),
           "value": round(npix / (statistics.mean(mar) * 1e-3) / 1e6, 2), "unit": "Mpix/s (march)",
           "stages_ms": {"voxelize": round(statistics.mean(vox), 4), "march": round(statistics.mean(mar), 4),
                         "blur": round(statistics.mean(blr), 4)},
           "request_mpix_s": round(npix / ((statistics.mean(vox) + statistics.mean(mar) + statistics.mean(blr)) * 1e-3)
                                   / 1e6, 2),
           "image": {"mean_rgb": round(float(img.mean()), 6)}}
    gi.close()
    return res


def run_batched(args, cfg=BATCHED):
    """Batched form: 64 resident scenes of mixed grid and triangle counts, 1-8 views each, all traces in one
    launch replayed from a CUDA graph (kernel variant tuned on the first batch)."""
    import math

    import numpy as np
    import torch

    import final184_gb300 as g

    rng = np.random.default_rng(cfg["seed"])
    dev = torch.device("cuda", 0)
    srv = g.Server(0, slots=1, max_batch_views=1024)
    gi = g.VoxelGI(0)
    reqs, keep, pixels, tris_total = [], [], 0, 0
    for k in range(cfg["scenes"]):
        dim = int(rng.choice(cfg["dims"]))
        ntris = int(math.exp(rng.uniform(math.log(cfg["tris"][0]), math.log(cfg["tris"][1]))))
        sc = g.SyntheticScene(cfg["seed"] + 17 * k, ntris, max(20, ntris // 250))
        tris_total += sc.ntris
        levels = int(math.log2(dim))
        srv.add_scene(k, g.GridDesc(dim, levels, g.FMT_F16, 0, min(2048, dim * 16), 0), sc.tri_xyz, sc.albedo,
                      sc.bounds, sc.light)
        tri = torch.from_numpy(sc.tri_xyz).to(dev)
        rough = torch.from_numpy(sc.roughness).to(dev)
        views = []
        for v in range(int(rng.integers(cfg["views"][0], cfg["views"][1] + 1))):
            (w0, h0), (w1, h1) = cfg["sizes"]
            t = rng.uniform(0, 1)
            W, H = int(w0 + t * (w1 - w0)), int(h0 + t * (h1 - h0))
            eye, tgt = sc.camera(v)
            Vm, Pm = g.look_at(eye, tgt), g.perspective(59.0, W / H, 0.1, 100.0)
            n = W * H
            bufs = (torch.empty(n, dtype=torch.float32, device=dev), torch.empty(n, dtype=torch.int32, device=dev),
                    torch.empty(n, dtype=torch.int16, device=dev), torch.empty(n * 8, dtype=torch.float16, device=dev))
            view = g.make_view(Vm, Pm, W, H, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(),
                               bufs[3].data_ptr(), g.FMT_F16)
            gi.gbuffer(tri.data_ptr(), rough.data_ptr(), sc.ntris, view)
            keep.append(bufs)
            views.append(view)
            pixels += n
        reqs.append((k, views, []))
        del tri, rough
    gi.sync()
    gi.close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first = [srv.wait(t) for t in srv.submit_many(reqs)]  # first batch: tunes the kernel variant
    first_s = time.perf_counter() - t0
    runs = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        res = [srv.wait(t) for t in srv.submit_many(reqs)]
        runs.append(time.perf_counter() - t0)
    st = srv.stats()
    srv.close()
    wall = statistics.median(runs)
    nviews = sum(len(v) for _, v, _ in reqs)
    lat = sorted(r.latency_ms for r in res)
    return {"workload": "%d resident scenes (grids %s^3, %.1fM triangles in all), %d views of 256^2..1920x1080, "
                        "FP16 storage, all traces in one launch per batch under a CUDA graph"
                        % (cfg["scenes"], "/".join(str(d) for d in cfg["dims"]), tris_total / 1e6, nviews),
            "value": round(pixels / wall / 1e6, 2), "unit": "Mpix/s", "pixels": int(pixels), "views": nviews,
            "batches_per_submit": len({r.batch for r in res}), "wall_ms": round(wall * 1e3, 3),
            "p50_ms": round(lat[len(lat) // 2], 3), "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * len(lat)))], 3),
            "first_batch_ms_with_tuning": round(first_s * 1e3, 1),
            "tuned": {"variant": int(st.trace_variant), "tile": [int(st.trace_tile[0]), int(st.trace_tile[1])],
                      "ctas_per_sm": int(st.trace_ctas_per_sm),
                      "tune_ms": [round(float(st.tune_ms[i]), 3) for i in range(st.trace_variants)]},
            "first_batch_status": sorted({r.status for r in first})}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="the 20k-triangle 64^3 640x360 case (profiling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="skip the served-vs-plain request stream")
    ap.add_argument("--no-precision", action="store_true", help="skip the 512^3 anisotropic FP16 precision form")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched form")
    ap.add_argument("--no-march", action="store_true", help="skip the reference-faithful march mode")
    ap.add_argument("--storage", choices=["f32", "f16"], default="f32",
                    help="grid storage of the plain leg (f32, the headline; f16 is the served form's storage)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    cfg = SMALL if args.small else PLAIN_LARGE
    if args.impl == "reference":  # the CPU restatement alone: the CUDA library is neither built nor loaded
        line = run_reference(args, cfg)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    from final184_gb300 import build as b

    b.build()
    rank, world, _ = dist_env()
    line, sc = run_gpu(args, cfg)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import build as ob

        ob.build_oracle()
        stride = 1  # the whole request: voxelization, mips and every row of the trace
        t, info, _ = cpu_request(cfg, stride, scene=sc)
        line["cpu_baseline"] = {
            "value": round(cfg["width"] * cfg["height"] / t / 1e6, 4), "unit": "Mpix/s", "cores": os.cpu_count(),
            "kind": "port",
            "sample": "one whole request on the CPU: shadow raster + voxelization + mip chain (%.1f s) and the cone trace "
                      "of all %d rows (%.1f s); FP32 restatement, std::thread over all cores"
                      % (info["voxelize_mip_s"], cfg["height"], info["trace_s"])}
        # the plain-small configuration is defined as a CPU run: the FP32 restatement of the whole request
        small = dict(SMALL, name="plain-small")
        ts, sinfo, _ = cpu_request(small, 1)
        line["plain_small_cpu"] = {
            "workload": workload_desc(small), "value": round(small["width"] * small["height"] / ts / 1e6, 4),
            "unit": "Mpix/s", "ms_per_request": round(ts * 1e3, 2), "cores": os.cpu_count(), "kind": "port",
            "note": "the FP32 CPU transcription of the path (oracle.cpp), all host threads: shadow raster + "
                    "voxelization + mips %.1f ms, trace of all %d rows %.1f ms"
                    % (sinfo["voxelize_mip_s"] * 1e3, small["height"], sinfo["trace_s"] * 1e3)}
    if rank == 0 and world == 1 and not args.no_served and not args.small:
        line["served"] = run_served(args)
    if rank == 0 and world == 1 and not args.no_batched and not args.small:
        line["batched"] = run_batched(args)
    if rank == 0 and world == 1 and not args.no_precision and not args.small:
        line["precision"] = run_precision(args)
    if rank == 0 and world == 1 and not args.no_march and not args.small:
        line["march"] = run_march(args)
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
