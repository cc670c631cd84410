// trace.cu -- host side of the cone trace: view tables, launches of the kernel variants (trace_kernel.cuh, one
// translation unit per storage format and mip kind), the batched launch under CUDA graphs (all views of a batch
// in one kernel), and the variant tuner.
#include <algorithm>
#include <vector>

#include "gi_internal.h"

namespace f184 {

const void* trace_kernel_f32_iso(uint32_t variant);
const void* trace_kernel_f32_aniso(uint32_t variant);
const void* trace_kernel_f16_iso(uint32_t variant);
const void* trace_kernel_f16_aniso(uint32_t variant);
const void* trace_kernel_count_f32_iso();
const void* trace_kernel_count_f32_aniso();
const void* trace_kernel_count_f16_iso();
const void* trace_kernel_count_f16_aniso();

const void* trace_kernel_fn(uint32_t fmt, bool aniso, uint32_t variant) {
    if (variant >= kTraceVariantCount) return nullptr;
    if (fmt == F184GI_FMT_F32) return aniso ? trace_kernel_f32_aniso(variant) : trace_kernel_f32_iso(variant);
    return aniso ? trace_kernel_f16_aniso(variant) : trace_kernel_f16_iso(variant);
}

const void* trace_kernel_count_fn(uint32_t fmt, bool aniso) {
    if (fmt == F184GI_FMT_F32) return aniso ? trace_kernel_count_f32_aniso() : trace_kernel_count_f32_iso();
    return aniso ? trace_kernel_count_f16_aniso() : trace_kernel_count_f16_iso();
}

uint32_t trace_view_tiles(uint32_t width, uint32_t height, uint32_t variant) {
    const TraceVariant& v = kTraceVariants[variant];
    const uint32_t wh = 32 / v.tw;  // warp tiles of tw x (32 / tw) pixels
    return ((width + v.tw - 1) / v.tw) * ((height + wh - 1) / wh);
}

void trace_view_set_grid(TraceView& v, const ChainLayout& c, const f184gi_grid_frame* d_frame, float tmax) {
    v.grid_base = c.base;
    v.grid_dim = c.dim;
    v.grid_levels = c.levels;
    v.frame = d_frame;
    v.tmax = tmax;
    for (int l = 0; l < kMaxLevels; ++l) {
        v.off[l] = l < int(c.levels) ? c.off[l] : 0;
        v.vol[l] = l < int(c.levels) ? c.vol[l] : 0;
    }
}

namespace {

// Table layout (host and device): [tile_base: nviews + 1 u32, padded to 256 B][views: nviews]
size_t table_header(uint32_t nviews) { return (size_t(nviews + 1) * 4 + 255) / 256 * 256; }
size_t table_bytes(uint32_t nviews) { return table_header(nviews) + size_t(nviews) * sizeof(TraceView); }

uint32_t fill_table(const TraceView* views, uint32_t nviews, uint32_t variant, unsigned char* h) {
    uint32_t* hb = reinterpret_cast<uint32_t*>(h);
    TraceView* hv = reinterpret_cast<TraceView*>(h + table_header(nviews));
    uint32_t tiles = 0;
    for (uint32_t i = 0; i < nviews; ++i) {
        hv[i] = views[i];
        hb[i] = tiles;
        tiles += trace_view_tiles(views[i].width, views[i].height, variant);
    }
    hb[nviews] = tiles;
    return tiles;
}

cudaError_t launch(const void* fn, uint32_t variant, uint32_t blocks, const TraceConsts& tc, const unsigned char* d_table,
                   uint32_t nviews, uint32_t* work, cudaStream_t s) {
    TraceConsts tcv = tc;
    const TraceView* dv = reinterpret_cast<const TraceView*>(d_table + table_header(nviews));
    const uint32_t* db = reinterpret_cast<const uint32_t*>(d_table);
    void* args[5] = {&tcv, &dv, &db, &nviews, &work};
    const TraceVariant& v = kTraceVariants[variant];
    return cudaLaunchKernel(fn, dim3(blocks), dim3(v.tw * v.th), args, 0, s);
}

}  // namespace

// Pinned host staging of the view table of the one-shot launch: reused once the event of its last copy has
// passed, so a launch never waits for the stream.
struct TraceStaging {
    unsigned char* host = nullptr;
    size_t bytes = 0;
    cudaEvent_t copied = nullptr;
};

void trace_staging_destroy(TraceStaging* st) {
    if (!st) return;
    if (st->copied) {
        cudaEventSynchronize(st->copied);
        cudaEventDestroy(st->copied);
    }
    cudaFreeHost(st->host);
    delete st;
}

size_t trace_scratch_bytes(uint32_t nviews) { return table_bytes(nviews) + 256; }

int trace_launch(const ChainLayout& c, const TraceConsts& tc, const f184gi_grid_frame* d_frame, const TraceView* views,
                 uint32_t nviews, void* scratch, size_t scratch_bytes, uint32_t variant, TraceStaging** staging,
                 cudaStream_t s, bool count) {
    if (nviews == 0) return F184GI_OK;
    if (scratch_bytes < trace_scratch_bytes(nviews)) return fail(F184GI_ERR_INVALID, "trace: scratch too small");
    if (count) variant = trace_default_variant(c.format, c.aniso != 0);
    const void* fn = count ? trace_kernel_count_fn(c.format, c.aniso != 0) : trace_kernel_fn(c.format, c.aniso != 0, variant);
    if (!fn) return fail(F184GI_ERR_INVALID, "trace: unknown kernel variant");
    const size_t need = table_bytes(nviews);
    TraceStaging* st = *staging;
    cudaError_t e = cudaSuccess;
    if (!st) {
        st = *staging = new TraceStaging();
        if ((e = cudaEventCreateWithFlags(&st->copied, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(e, "trace: staging event");
    }
    if ((e = cudaEventSynchronize(st->copied)) != cudaSuccess) return cuda_fail(e, "trace: staging wait");
    if (st->bytes < need) {
        cudaFreeHost(st->host);
        st->host = nullptr;
        st->bytes = 0;
        if ((e = cudaHostAlloc(&st->host, need, cudaHostAllocDefault)) != cudaSuccess)
            return cuda_fail(e, "trace: staging allocation");
        st->bytes = need;
    }
    std::vector<TraceView> vv(views, views + nviews);
    for (auto& v : vv) trace_view_set_grid(v, c, d_frame, tc.tmax);
    const uint32_t tiles = fill_table(vv.data(), nviews, variant, st->host);
    unsigned char* d_table = static_cast<unsigned char*>(scratch);
    if ((e = cudaMemcpyAsync(d_table, st->host, need, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "trace: view table");
    if ((e = cudaEventRecord(st->copied, s)) != cudaSuccess) return cuda_fail(e, "trace: staging event");
    if (tiles == 0) return F184GI_OK;
    const uint32_t warps = kTraceVariants[variant].tw * kTraceVariants[variant].th / 32;
    e = launch(fn, variant, (tiles + warps - 1) / warps, tc, d_table, nviews, nullptr, s);
    note_launches(1);
    return cuda_fail(e, "trace");
}

// ---------------- batched trace under CUDA graphs ----------------

// One graph per kernel variant, instantiated on first use:
//   [view table H2D] -> [work counter = 0] -> [kernel: one warp per warp tile, or a capped persistent wave]
struct TraceGraphVariant {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t copy = nullptr, reset = nullptr, kernel = nullptr;
    uint32_t blocks = 0;
};

struct TraceGraph {
    uint32_t fmt = 0;
    bool aniso = false;
    uint32_t max_views = 0, per_sm = 0;
    size_t bytes = 0;
    unsigned char* h_table = nullptr;
    unsigned char* d_table = nullptr;
    uint32_t* d_work = nullptr;
    TraceConsts tc{};
    uint32_t nviews = 0;
    const TraceView* kviews = nullptr;
    const uint32_t* kbase = nullptr;
    uint32_t* kwork = nullptr;  // null: static warp tiles
    uint32_t tiles = 0;         // warp tiles of the current batch
    TraceGraphVariant var[kTraceVariantCount];
};

uint32_t trace_persistent_blocks(uint32_t fmt, bool aniso, uint32_t variant, uint32_t per_sm) {
    int dev = 0, sms = 0, maxb = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const TraceVariant& v = kTraceVariants[variant];
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, trace_kernel_fn(fmt, aniso, variant), int(v.tw * v.th), 0);
    if (maxb <= 0) maxb = 1;
    uint32_t b = per_sm ? std::min<uint32_t>(per_sm, uint32_t(maxb)) : uint32_t(maxb);
    return b * uint32_t(sms > 0 ? sms : 1);
}

static void graph_params(TraceGraph* g, uint32_t variant, cudaKernelNodeParams& kp, void** args) {
    args[0] = &g->tc;
    args[1] = &g->kviews;
    args[2] = &g->kbase;
    args[3] = &g->nviews;
    args[4] = &g->kwork;
    const TraceVariant& v = kTraceVariants[variant];
    kp = cudaKernelNodeParams{};
    kp.func = const_cast<void*>(trace_kernel_fn(g->fmt, g->aniso, variant));
    // per_sm 0: every warp tile of the batch gets its own warp (the hardware block scheduler balances the views;
    // measured as fast as a persistent wave).  per_sm > 0: a persistent wave of per_sm CTAs per SM whose warps
    // take tiles from the work counter, leaving the rest of each SM to other work.
    const uint32_t warps = v.tw * v.th / 32;
    g->kwork = g->per_sm ? g->d_work : nullptr;
    kp.gridDim = dim3(g->per_sm ? g->var[variant].blocks : std::max<uint32_t>(1u, (g->tiles + warps - 1) / warps));
    kp.blockDim = dim3(v.tw * v.th);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
}

static cudaError_t graph_variant(TraceGraph* g, uint32_t variant) {
    TraceGraphVariant& gv = g->var[variant];
    if (gv.exec) return cudaSuccess;
    gv.blocks = trace_persistent_blocks(g->fmt, g->aniso, variant, g->per_sm);
    cudaError_t e = cudaGraphCreate(&gv.graph, 0);
    if (e == cudaSuccess)
        e = cudaGraphAddMemcpyNode1D(&gv.copy, gv.graph, nullptr, 0, g->d_table, g->h_table, g->bytes,
                                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        cudaMemsetParams mp{};
        mp.dst = g->d_work;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = 1;
        mp.height = 1;
        mp.pitch = 4;
        e = cudaGraphAddMemsetNode(&gv.reset, gv.graph, &gv.copy, 1, &mp);
    }
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp;
        void* args[5];
        g->nviews = g->max_views;
        g->kbase = reinterpret_cast<const uint32_t*>(g->d_table);
        g->kviews = reinterpret_cast<const TraceView*>(g->d_table + table_header(g->max_views));
        graph_params(g, variant, kp, args);
        e = cudaGraphAddKernelNode(&gv.kernel, gv.graph, &gv.reset, 1, &kp);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&gv.exec, gv.graph, 0);
    return e;
}

int trace_graph_create(TraceGraph** out, uint32_t fmt, bool aniso, uint32_t max_views, uint32_t per_sm,
                       const TraceConsts& tc) {
    *out = nullptr;
    TraceGraph* g = new TraceGraph();
    g->fmt = fmt, g->aniso = aniso, g->max_views = max_views, g->per_sm = per_sm, g->tc = tc;
    g->bytes = table_bytes(max_views);
    cudaError_t e = cudaHostAlloc(&g->h_table, g->bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_table, g->bytes + 256);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_work, 256);
    if (e != cudaSuccess) {
        trace_graph_destroy(g);
        return cuda_fail(e, "trace graph");
    }
    *out = g;
    return F184GI_OK;
}

// The table is laid out for this batch's view count; the kernel node gets pointers into it.
int trace_graph_launch(TraceGraph* g, const TraceView* views, uint32_t nviews, uint32_t variant, cudaStream_t s) {
    if (nviews == 0) return F184GI_OK;
    if (nviews > g->max_views) return fail(F184GI_ERR_INVALID, "trace graph: batch exceeds max_views");
    if (variant >= kTraceVariantCount) return fail(F184GI_ERR_INVALID, "trace graph: unknown variant");
    cudaError_t e = graph_variant(g, variant);
    if (e != cudaSuccess) return cuda_fail(e, "trace graph");
    TraceGraphVariant& gv = g->var[variant];
    g->tiles = fill_table(views, nviews, variant, g->h_table);
    g->nviews = nviews;
    g->kbase = reinterpret_cast<const uint32_t*>(g->d_table);
    g->kviews = reinterpret_cast<const TraceView*>(g->d_table + table_header(nviews));
    e = cudaGraphExecMemcpyNodeSetParams1D(gv.exec, gv.copy, g->d_table, g->h_table, table_bytes(nviews),
                                           cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        cudaKernelNodeParams kp;
        void* args[5];
        graph_params(g, variant, kp, args);
        e = cudaGraphExecKernelNodeSetParams(gv.exec, gv.kernel, &kp);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(gv.exec, s);
    if (e == cudaSuccess) note_launches(1);
    return cuda_fail(e, "trace graph launch");
}

// Self-tuning: trace this batch once with every variant (each run writes the same outputs), twice over, and
// keep the variant with the shortest time.  The batch runs alone on the device while it is tuned.
int trace_graph_tune(TraceGraph* g, const TraceView* views, uint32_t nviews, cudaStream_t s, uint32_t* best,
                     float* ms_out) {
    cudaEvent_t ev[2];
    cudaError_t e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    if (e != cudaSuccess) return cuda_fail(e, "trace tune: events");
    float ms[kTraceVariantCount];
    int rc = F184GI_OK;
    for (uint32_t v = 0; v < kTraceVariantCount; ++v) ms[v] = 3.0e38f;
    for (int round = 0; round < 2 && rc == F184GI_OK; ++round)
        for (uint32_t v = 0; v < kTraceVariantCount && rc == F184GI_OK; ++v) {
            // the host table is rewritten per variant: the previous run (and its copy) must be complete
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {
                rc = cuda_fail(e, "trace tune");
                break;
            }
            cudaEventRecord(ev[0], s);
            if ((rc = trace_graph_launch(g, views, nviews, v, s))) break;
            cudaEventRecord(ev[1], s);
            if ((e = cudaEventSynchronize(ev[1])) != cudaSuccess) {
                rc = cuda_fail(e, "trace tune");
                break;
            }
            float t = 0.0f;
            cudaEventElapsedTime(&t, ev[0], ev[1]);
            ms[v] = std::min(ms[v], t);
        }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rc) return rc;
    uint32_t b = 0;
    for (uint32_t v = 1; v < kTraceVariantCount; ++v)
        if (ms[v] < ms[b]) b = v;
    *best = b;
    if (ms_out)
        for (uint32_t v = 0; v < kTraceVariantCount; ++v) ms_out[v] = ms[v];
    return F184GI_OK;
}

void trace_graph_destroy(TraceGraph* g) {
    if (!g) return;
    for (TraceGraphVariant& gv : g->var) {
        if (gv.exec) cudaGraphExecDestroy(gv.exec);
        if (gv.graph) cudaGraphDestroy(gv.graph);
    }
    cudaFreeHost(g->h_table);
    cudaFree(g->d_table);
    cudaFree(g->d_work);
    delete g;
}

}  // namespace f184
