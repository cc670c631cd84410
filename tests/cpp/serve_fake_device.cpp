// serve_fake_device.cpp -- a host-only stand-in for the CUDA runtime and for the f184gi calls the request server
// (final184_gb300/csrc/serve.cpp) makes, so that the server's threads can run under ThreadSanitizer on a CPU.
//
// Streams are modelled as queues of work with a completion time: every call that would issue device work adds a
// short delay to its stream, an event recorded on a stream completes when the stream's queued work does, and
// synchronising on an event or stream sleeps until then.  Device memory is host memory.  The fake keeps its own
// state under one mutex, so anything ThreadSanitizer reports is the server's.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>

#include "../../final184_gb300/csrc/gi_internal.h"

namespace {
using Clock = std::chrono::steady_clock;
std::mutex g_mu;
std::map<void*, Clock::time_point> g_stream_done;  // stream -> when its queued work is done
std::map<void*, Clock::time_point> g_event_done;
int g_stream_id = 0, g_event_id = 0;
thread_local int g_device = 0;

void add_work(cudaStream_t s, int us) {
    std::lock_guard<std::mutex> lk(g_mu);
    Clock::time_point& t = g_stream_done[s];
    const Clock::time_point now = Clock::now();
    if (t < now) t = now;
    t += std::chrono::microseconds(us);
}
void sleep_until(Clock::time_point t) { std::this_thread::sleep_until(t); }
}  // namespace

struct f184gi_ctx {
    int device;
};

extern "C" {
cudaError_t cudaSetDevice(int d) { g_device = d; return cudaSuccess; }
cudaError_t cudaGetDevice(int* d) { *d = g_device; return cudaSuccess; }
cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr, int) { *v = 152; return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) {
    Clock::time_point last = Clock::now();
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (auto& kv : g_stream_done) last = std::max(last, kv.second);
    }
    sleep_until(last);
    return cudaSuccess;
}
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned int) {
    std::lock_guard<std::mutex> lk(g_mu);
    *s = reinterpret_cast<cudaStream_t>(new int(++g_stream_id));
    g_stream_done[*s] = Clock::now();
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_stream_done.erase(s);
    delete reinterpret_cast<int*>(s);
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t s) {
    Clock::time_point t;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        t = g_stream_done[s];
    }
    sleep_until(t);
    return cudaSuccess;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int) {
    std::lock_guard<std::mutex> lk(g_mu);
    *e = reinterpret_cast<cudaEvent_t>(new int(++g_event_id));
    g_event_done[*e] = Clock::now();
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_event_done.erase(e);
    delete reinterpret_cast<int*>(e);
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(g_mu);
    const Clock::time_point now = Clock::now();
    Clock::time_point t = g_stream_done[s];
    g_event_done[e] = t < now ? now : t;
    return cudaSuccess;
}
cudaError_t cudaStreamWaitEvent(cudaStream_t s, cudaEvent_t e, unsigned int) {
    // the stream's later work starts after the event's: its completion time moves past the event's
    std::lock_guard<std::mutex> lk(g_mu);
    const Clock::time_point te = g_event_done[e];
    Clock::time_point& t = g_stream_done[s];
    if (t < te) t = te;
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t e) {
    Clock::time_point t;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        t = g_event_done[e];
    }
    sleep_until(t);
    return cudaSuccess;
}
cudaError_t cudaMalloc(void** p, size_t n) { *p = std::calloc(1, n ? n : 1); return *p ? cudaSuccess : cudaErrorMemoryAllocation; }
cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
cudaError_t cudaHostAlloc(void** p, size_t n, unsigned int) { return cudaMalloc(p, n); }
cudaError_t cudaFreeHost(void* p) { std::free(p); return cudaSuccess; }
cudaError_t cudaMallocAsync(void** p, size_t n, cudaStream_t s) { add_work(s, 5); return cudaMalloc(p, n); }
cudaError_t cudaFreeAsync(void* p, cudaStream_t s) {
    // the block is released once the stream's queued work is done: a real stream-ordered free
    cudaStreamSynchronize(s);
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return cudaSuccess; }
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t st) {
    std::memcpy(d, s, n);  // copies at issue: the server does not rewrite a source before its copy is ordered
    add_work(st, 10);
    return cudaSuccess;
}

int f184gi_create(const f184gi_config* cfg, f184gi_ctx** out) {
    *out = new f184gi_ctx{cfg ? cfg->device : 0};
    return F184GI_OK;
}
int f184gi_destroy(f184gi_ctx* c) { delete c; return F184GI_OK; }
int f184gi_grid_bytes(const f184gi_grid_desc* d, uint64_t* b) { *b = uint64_t(d->dim) * d->dim * d->dim * 8; return F184GI_OK; }
int f184gi_grid_create(f184gi_ctx*, const f184gi_grid_desc*, uint32_t* g) { *g = 1; return F184GI_OK; }
int f184gi_voxelize(f184gi_ctx*, uint32_t, const float*, const uint32_t*, uint64_t, const f184gi_bounds*,
                    const f184gi_light*, const uint32_t*, uint32_t, void* s) {
    add_work(static_cast<cudaStream_t>(s), 200);
    return F184GI_OK;
}
int f184gi_mip(f184gi_ctx*, uint32_t, uint32_t, uint32_t, void* s) { add_work(static_cast<cudaStream_t>(s), 50); return F184GI_OK; }
int f184gi_apply_moves(f184gi_ctx*, float*, const f184gi_move*, uint32_t, uint64_t, void* s) {
    add_work(static_cast<cudaStream_t>(s), 10);
    return F184GI_OK;
}
int f184gi_sync(f184gi_ctx*, void* s) { return cudaStreamSynchronize(static_cast<cudaStream_t>(s)) == cudaSuccess ? F184GI_OK : F184GI_ERR_CUDA; }
void f184gi_cone_params_default(f184gi_cone_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->diffuse_cones = 5;
    p->diffuse_tan_half = 0.57735026f;
    p->diffuse_tilt_deg = 60.0f;
    p->step_factor = 0.5f;
    p->alpha_stop = 1.0f;
    p->start_offset = 1.0f;
    p->min_spec_tan_half = 0.05f;
    p->specular = 1;
}
}  // extern "C"

namespace f184 {
struct TraceGraph {
    int dummy;
};
int fail(int code, const std::string&) { return code; }
int cuda_fail(cudaError_t e, const char*) { return e == cudaSuccess ? F184GI_OK : F184GI_ERR_CUDA; }
bool invert4(const double* m, double* inv) {
    for (int k = 0; k < 16; ++k) inv[k] = m[k];
    return true;
}
int compute_frame(const f184gi_bounds&, uint32_t, const float*, f184gi_grid_frame* out) {
    std::memset(out, 0, sizeof(*out));
    out->voxel_size = 0.1;
    return F184GI_OK;
}
int grid_internal(f184gi_ctx*, uint32_t, ChainLayout* chain, const f184gi_grid_frame** d_frame) {
    std::memset(chain, 0, sizeof(*chain));
    *d_frame = nullptr;
    return F184GI_OK;
}
size_t raster_scratch_bytes(uint64_t ntris, uint32_t, uint32_t) { return ntris * 48; }
size_t voxelize_scratch_bytes(uint64_t ntris, uint32_t) { return ntris * 64; }
void trace_consts_schedule(TraceConsts&) {}
uint32_t trace_persistent_blocks(uint32_t, bool, uint32_t, uint32_t) { return 152 * 5; }
void trace_view_set_grid(TraceView& v, const ChainLayout&, const f184gi_grid_frame*, float tmax) { v.tmax = tmax; }
int trace_graph_create(TraceGraph** out, uint32_t, bool, uint32_t, uint32_t, const TraceConsts&) {
    *out = new TraceGraph{0};
    return F184GI_OK;
}
int trace_graph_launch(TraceGraph*, const TraceView*, uint32_t nviews, uint32_t, cudaStream_t s) {
    add_work(s, 100 + 20 * int(nviews));
    return F184GI_OK;
}
int trace_graph_tune(TraceGraph* g, const TraceView* v, uint32_t n, cudaStream_t s, uint32_t* best, float* ms) {
    for (uint32_t k = 0; k < kTraceVariantCount; ++k) ms[k] = 1.0f + float(k);
    *best = 0;
    return trace_graph_launch(g, v, n, 0, s);
}
void trace_graph_destroy(TraceGraph* g) { delete g; }
int ctx_status_capture(f184gi_ctx*, uint32_t* host_pinned, cudaStream_t s) {
    *host_pinned = 0;  // the fake's kernels raise no flags
    add_work(s, 2);
    return F184GI_OK;
}
int ctx_status_report(f184gi_ctx*, uint32_t status) { return status ? F184GI_ERR_INVALID : F184GI_OK; }
}  // namespace f184
