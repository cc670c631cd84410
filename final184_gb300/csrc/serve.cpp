// serve.cpp -- the served form: continuous batching of GI requests over device-resident scenes.
//
// The reference renders one frame at a time from one render thread (App/Game.cpp:248-345, CMegaPipeline::Render);
// this host runtime instead serves a stream of requests (object moves + view sets) against scenes kept on the
// device.  A scheduler thread forms batches whenever one of `slots` in-flight batches is free:
//   - admission: one request per scene per batch (a scene's requests apply in submission order), the HBM budget
//     for staging of host-buffer requests, at most max_batch_views views;
//   - per touched scene: rigid moves on the device, dirty bricks from the moved objects' old and new boxes
//     (computed on a host mirror of the geometry), geometry re-voxelization of those bricks, relight of the grid
//     from the new shadow map, mip rebuild;
//   - one trace launch over all views of the batch, replayed from the slot's CUDA graph.
// A completer thread retires batches in launch order and records per-request latency.  Batches on different
// slots overlap on the device; requests that arrive meanwhile join the next batch.
// Failures are per request: a request whose staging, update or view set-up fails finishes with that status and the
// rest of its batch runs.  If the scheduler thread stops (for any reason, or by the INJECT_WORKER_EXIT test hook),
// its exit path fails the batch it was forming and every queued request with F184GI_ERR_WORKER and the server
// refuses new requests, so no caller waits on a request nothing will run.
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

#include "gi_internal.h"

using namespace f184;

namespace {

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Scene {
    uint32_t id = 0;
    f184gi_ctx* ctx = nullptr;
    uint32_t grid = 0;
    f184gi_grid_desc desc{};
    float* d_tri = nullptr;
    uint32_t* d_alb = nullptr;
    uint64_t ntris = 0;
    std::vector<float> h_tri;  // host mirror of the device geometry (same FP32 adds)
    f184gi_bounds bounds{};
    f184gi_light light{};
    f184gi_grid_frame frame{};
    ChainLayout chain{};
    const f184gi_grid_frame* d_frame = nullptr;
    uint32_t* d_dirty = nullptr;
    uint32_t* h_dirty = nullptr;  // pinned staging of the dirty list
    uint32_t nbricks = 0;
    std::vector<uint8_t> flag;
    // Batches in flight that hold this scene (one request each, in admission order) and the slot of the latest:
    // a later batch's update of the scene waits on that slot's completion event, so the scene's requests run in
    // order without one in flight blocking the next one's admission.
    uint32_t inflight = 0;
    int last_slot = -1;
    cudaEvent_t dirty_copied = nullptr;  // the last update's copy of h_dirty has been made (h_dirty reusable)
    uint64_t bytes = 0;
};

struct Request {
    uint64_t ticket = 0;
    uint32_t scene = 0, flags = 0;
    std::vector<f184gi_move> moves;
    std::vector<f184gi_view> views;   // as submitted
    Clock::time_point t_submit, t_admit, t_done;
    int status = 0;
    bool done = false, admitted = false;
    uint32_t batch = 0;
    uint64_t pixels = 0, staging = 0;
    void* d_stage = nullptr;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    TraceGraph* graph = nullptr;
    std::vector<Request*> reqs;
    std::vector<int> req_status;  // per request: a failure of its own staging / update / views (0 = ran)
    std::vector<Scene*> scenes;  // scene of each request, resolved under the server lock
    std::vector<cudaEvent_t> waits;  // per request: completion event of the scene's previous batch (or null)
    uint32_t* h_status = nullptr;    // pinned: each scene context's status word, captured at the end of the batch
    std::vector<TraceView> tv;
    uint32_t batch = 0;
    bool busy = false;
};

uint64_t staging_bytes(const f184gi_request& r) {
    if (!(r.flags & F184GI_REQ_HOST_BUFFERS)) return 0;
    uint64_t b = 0;
    for (uint32_t i = 0; i < r.nviews; ++i) {
        uint64_t n = uint64_t(r.views[i].width) * r.views[i].height;
        uint64_t out = r.views[i].out_format == F184GI_FMT_F32 ? 32 : 16;
        b += ((n * (4 + 4 + 2 + out)) + 1023) / 1024 * 1024;
    }
    return b;
}

}  // namespace

struct f184gi_server {
    f184gi_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::deque<Request*> pending;
    std::map<uint64_t, Request*> reqs;
    std::map<uint32_t, Scene*> scenes;
    std::vector<Slot> slots;
    std::deque<int> launched;
    std::thread sched, completer;
    bool stop = false;
    bool worker_lost = false;  // the scheduler thread has stopped while the server was running
    FILE* log = nullptr;       // per-request JSON lines (f184gi_server_set_log)
    uint64_t next_ticket = 1, generation = 0;
    uint32_t next_batch = 1;
    uint64_t hbm_used = 0;
    int fmt = -1, aniso = -1;
    TraceConsts tc{};
    int variant = -1;  // trace kernel variant, tuned on the first batch
    float tune_ms[kTraceVariantCount] = {};
    std::vector<double> lat;
    uint64_t done_n = 0, cancelled = 0, batches = 0, pixels = 0, batch_views = 0;
};

namespace {

uint32_t sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return uint32_t(sms > 0 ? sms : 1);
}

void mark_box(Scene* sc, const float mn[3], const float mx[3]) {
    const double vs = sc->frame.voxel_size;
    const int dim = int(sc->desc.dim);
    int b0[3], b1[3];
    for (int a = 0; a < 3; ++a) {
        // conservative: one voxel of margin around the closed box
        double lo = std::floor((double(mn[a]) - sc->frame.origin[a]) / vs) - 1.0;
        double hi = std::floor((double(mx[a]) - sc->frame.origin[a]) / vs) + 1.0;
        int i0 = int(std::max(0.0, std::min(double(dim - 1), lo)));
        int i1 = int(std::max(0.0, std::min(double(dim - 1), hi)));
        b0[a] = i0 >> 3, b1[a] = i1 >> 3;
    }
    for (int z = b0[2]; z <= b1[2]; ++z)
        for (int y = b0[1]; y <= b1[1]; ++y)
            for (int x = b0[0]; x <= b1[0]; ++x) {
                uint32_t m = 0;
                for (int bit = 0; bit < 10; ++bit)
                    m |= (((uint32_t(x) >> bit) & 1u) << (3 * bit)) | (((uint32_t(y) >> bit) & 1u) << (3 * bit + 1)) |
                         (((uint32_t(z) >> bit) & 1u) << (3 * bit + 2));
                sc->flag[m] = 1;
            }
}

void range_box(const Scene* sc, uint32_t first, uint32_t count, float mn[3], float mx[3]) {
    for (int a = 0; a < 3; ++a) mn[a] = 1e30f, mx[a] = -1e30f;
    const float* p = sc->h_tri.data() + uint64_t(first) * 9;
    for (uint64_t v = 0; v < uint64_t(count) * 3; ++v)
        for (int a = 0; a < 3; ++a) {
            mn[a] = std::min(mn[a], p[v * 3 + a]);
            mx[a] = std::max(mx[a], p[v * 3 + a]);
        }
}

// Scene work of one request on `s`: moves, dirty-brick re-voxelization, relight, mips.
int scene_update(Scene* sc, const Request* r, cudaStream_t s) {
    if (r->moves.empty()) return F184GI_OK;
    std::fill(sc->flag.begin(), sc->flag.end(), 0);
    for (const f184gi_move& m : r->moves) {
        float mn[3], mx[3];
        range_box(sc, m.first, m.count, mn, mx);
        mark_box(sc, mn, mx);
        float* p = sc->h_tri.data() + uint64_t(m.first) * 9;
        for (uint64_t v = 0; v < uint64_t(m.count) * 3; ++v)
            for (int a = 0; a < 3; ++a) p[v * 3 + a] = p[v * 3 + a] + m.offset[a];
        range_box(sc, m.first, m.count, mn, mx);
        mark_box(sc, mn, mx);
    }
    // the previous update's copy of the dirty list may still be queued on another slot's stream
    cudaError_t e = cudaEventSynchronize(sc->dirty_copied);
    if (e != cudaSuccess) return cuda_fail(e, "server: dirty list reuse");
    uint32_t nd = 0;
    for (uint32_t m = 0; m < sc->nbricks; ++m)
        if (sc->flag[m]) sc->h_dirty[nd++] = m;
    int rc = f184gi_apply_moves(sc->ctx, sc->d_tri, r->moves.data(), uint32_t(r->moves.size()), sc->ntris, s);
    if (rc) return rc;
    if (nd == 0) return F184GI_OK;
    e = cudaMemcpyAsync(sc->d_dirty, sc->h_dirty, size_t(nd) * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(sc->dirty_copied, s);
    if (e != cudaSuccess) return cuda_fail(e, "server: dirty list");
    rc = f184gi_voxelize(sc->ctx, sc->grid, sc->d_tri, sc->d_alb, sc->ntris, &sc->bounds, &sc->light, sc->d_dirty, nd, s);
    if (rc) return rc;
    return f184gi_mip(sc->ctx, sc->grid, 0, sc->desc.anisotropic, s);
}

int prepare_view(f184gi_server* S, const Scene* sc, const f184gi_view& v, TraceView& t) {
    double V[16], P[16], IV[16], IP[16];
    for (int k = 0; k < 16; ++k) V[k] = v.view[k], P[k] = v.proj[k];
    if (!invert4(V, IV) || !invert4(P, IP)) return fail(F184GI_ERR_INVALID, "server: singular view or projection");
    t = TraceView{};
    trace_view_set_inverses(t, IP, IV);
    t.eye[0] = float(IV[3]), t.eye[1] = float(IV[7]), t.eye[2] = float(IV[11]);
    t.width = v.width, t.height = v.height;
    t.depth = v.depth, t.normal = v.normal, t.rough = v.roughness, t.out = v.out, t.out_format = v.out_format;
    float tmax = S->tc.p.max_distance > 0.0f ? S->tc.p.max_distance : float(double(sc->desc.dim) * std::sqrt(3.0));
    trace_view_set_grid(t, sc->chain, sc->d_frame, tmax);
    return F184GI_OK;
}

// Stage host-buffer request inputs on the device (allocation from the stream-ordered pool).
int stage_in(Request* r, cudaStream_t s) {
    if (!(r->flags & F184GI_REQ_HOST_BUFFERS)) return F184GI_OK;
    cudaError_t e = cudaMallocAsync(&r->d_stage, r->staging, s);
    if (e != cudaSuccess) return cuda_fail(e, "server: staging allocation");
    unsigned char* p = static_cast<unsigned char*>(r->d_stage);
    for (f184gi_view& v : r->views) {
        const uint64_t n = uint64_t(v.width) * v.height;
        const uint64_t out = v.out_format == F184GI_FMT_F32 ? 32 : 16;
        unsigned char* d_depth = p;
        unsigned char* d_norm = d_depth + n * 4;
        unsigned char* d_rough = d_norm + n * 4;
        unsigned char* d_out = d_rough + n * 2;
        p += ((n * (10 + out)) + 1023) / 1024 * 1024;
        if ((e = cudaMemcpyAsync(d_depth, v.depth, n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_norm, v.normal, n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(d_rough, v.roughness, n * 2, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail(e, "server: staging copy");
        v.depth = reinterpret_cast<const float*>(d_depth);
        v.normal = reinterpret_cast<const uint32_t*>(d_norm);
        v.roughness = reinterpret_cast<const uint16_t*>(d_rough);
        (void)out;
        // keep the caller's host output pointer in `pad`-sized side storage: swap after the trace
        v.out = d_out;
    }
    return F184GI_OK;
}

int stage_out(Request* r, const std::vector<void*>& host_out, cudaStream_t s) {
    if (!(r->flags & F184GI_REQ_HOST_BUFFERS)) return F184GI_OK;
    for (size_t i = 0; i < r->views.size(); ++i) {
        const f184gi_view& v = r->views[i];
        const uint64_t n = uint64_t(v.width) * v.height * (v.out_format == F184GI_FMT_F32 ? 32 : 16);
        cudaError_t e = cudaMemcpyAsync(host_out[i], v.out, n, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(e, "server: result copy");
    }
    cudaError_t e = cudaFreeAsync(r->d_stage, s);
    r->d_stage = nullptr;
    return cuda_fail(e, "server: staging free");
}

// NVTX range for the duration of a scope (visible in Nsight Systems / ncu's NVTX filter)
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

// The batch's device work on the slot's stream.  A request whose staging, scene update or view set-up fails gets
// that status in slot.req_status and its views are left out; the others run.  The return value is a failure of
// the batch itself (graph, launch, event), which fails every request of the batch.
int issue_batch(f184gi_server* S, Slot& slot) {
    NvtxRange range("f184gi server batch");
    cudaStream_t s = slot.stream;
    slot.tv.clear();
    slot.req_status.assign(slot.reqs.size(), F184GI_OK);
    std::vector<std::vector<void*>> host_out(slot.reqs.size());
    {
        NvtxRange r_update("f184gi server: staging + scene updates");
        for (size_t k = 0; k < slot.reqs.size(); ++k) {
            Request* r = slot.reqs[k];
            Scene* sc = slot.scenes[k];
            for (const f184gi_view& v : r->views) host_out[k].push_back(v.out);
            const size_t first_view = slot.tv.size();
            // the scene's previous batch (another slot) reads the grid its update is about to rewrite
            int rc = slot.waits[k] ? cuda_fail(cudaStreamWaitEvent(s, slot.waits[k], 0), "server: scene order") : 0;
            if (!rc)
                rc = (r->flags & F184GI_REQ_INJECT_FAIL)
                         ? fail(F184GI_ERR_CUDA, "server: injected failure of the scene update (test hook)")
                         : stage_in(r, s);
            if (!rc) rc = scene_update(sc, r, s);
            for (size_t v = 0; !rc && v < r->views.size(); ++v) {
                TraceView t;
                if (!(rc = prepare_view(S, sc, r->views[v], t))) slot.tv.push_back(t);
            }
            if (rc) {
                slot.req_status[k] = rc;
                slot.tv.resize(first_view);
                if (r->d_stage) {
                    cudaFreeAsync(r->d_stage, s);
                    r->d_stage = nullptr;
                }
            }
        }
    }
    int rc = F184GI_OK;
    if (!slot.tv.empty()) {
        NvtxRange r_trace("f184gi server: batched trace");
        if (!slot.graph) {
            rc = trace_graph_create(&slot.graph, uint32_t(S->fmt), S->aniso != 0, S->cfg.max_batch_views,
                                    S->cfg.blocks_per_sm, S->tc);
            if (rc) return rc;
        }
        if (S->variant < 0) {  // first batch: it runs alone (the scheduler issues nothing else meanwhile)
            uint32_t best = trace_default_variant(uint32_t(S->fmt), S->aniso != 0);
            float ms[kTraceVariantCount];
            if ((rc = trace_graph_tune(slot.graph, slot.tv.data(), uint32_t(slot.tv.size()), s, &best, ms))) return rc;
            std::lock_guard<std::mutex> lk(S->mu);
            for (uint32_t v = 0; v < kTraceVariantCount; ++v) S->tune_ms[v] = ms[v];
            S->variant = int(best);
        } else {
            rc = trace_graph_launch(slot.graph, slot.tv.data(), uint32_t(slot.tv.size()), uint32_t(S->variant), s);
            if (rc) return rc;
        }
    }
    for (size_t k = 0; k < slot.reqs.size(); ++k)
        if (slot.req_status[k] == F184GI_OK && (rc = stage_out(slot.reqs[k], host_out[k], s))) return rc;
    // each scene's status word, taken in stream order: flags raised by this batch's kernels are reported with
    // this batch, not with a later batch of the same scene that may run by the time this one is retired
    for (size_t k = 0; k < slot.scenes.size(); ++k)
        if ((rc = ctx_status_capture(slot.scenes[k]->ctx, slot.h_status + k, s))) return rc;
    return cuda_fail(cudaEventRecord(slot.done, s), "server: batch event");
}

int free_slot(f184gi_server* S) {
    for (size_t i = 0; i < S->slots.size(); ++i)
        if (!S->slots[i].busy) return int(i);
    return -1;
}

void finish_request(f184gi_server* S, Request* r, int status, Clock::time_point now) {
    r->status = status;
    r->done = true;
    r->t_done = now;
    if (status == F184GI_OK) {
        S->lat.push_back(ms_between(r->t_submit, now));
        S->done_n += 1;
        S->pixels += r->pixels;
    }
    S->hbm_used -= r->staging;
    if (S->log) {
        std::fprintf(S->log,
                     "{\"ticket\": %llu, \"scene\": %u, \"status\": %d, \"batch\": %u, \"views\": %zu, "
                     "\"moves\": %zu, \"pixels\": %llu, \"queued_ms\": %.3f, \"latency_ms\": %.3f}\n",
                     (unsigned long long)r->ticket, r->scene, status, r->batch, r->views.size(), r->moves.size(),
                     (unsigned long long)r->pixels, r->admitted ? ms_between(r->t_submit, r->t_admit) : 0.0,
                     ms_between(r->t_submit, now));
        std::fflush(S->log);
    }
}

// Runs when the scheduler thread leaves its loop for any reason.  Unless the server is being destroyed, the worker
// is lost: the batch it was forming (admitted, not issued) and every queued request fail with F184GI_ERR_WORKER,
// and later submissions are refused; batches already issued are still retired by the completer.
void scheduler_exit(f184gi_server* S) {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return;
    S->worker_lost = true;
    const Clock::time_point now = Clock::now();
    for (Slot& sl : S->slots) {
        if (!sl.busy || std::find(S->launched.begin(), S->launched.end(), int(&sl - S->slots.data())) != S->launched.end())
            continue;
        for (size_t k = 0; k < sl.reqs.size(); ++k) {
            finish_request(S, sl.reqs[k], F184GI_ERR_WORKER, now);
            sl.scenes[k]->inflight -= 1;
        }
        sl.reqs.clear();
        sl.busy = false;
    }
    for (Request* r : S->pending) finish_request(S, r, F184GI_ERR_WORKER, now);
    S->pending.clear();
    S->generation++;
    S->cv_done.notify_all();
}

void scheduler_loop(f184gi_server* S);

void scheduler(f184gi_server* S) {
    try {
        scheduler_loop(S);
    } catch (...) {  // e.g. a host allocation failure: the worker is lost, the exit path below reports it
    }
    scheduler_exit(S);
}

void scheduler_loop(f184gi_server* S) {
    cudaSetDevice(S->cfg.device);
    std::unique_lock<std::mutex> lk(S->mu);
    uint64_t seen = S->generation;
    while (true) {
        S->cv_sched.wait(lk, [&] { return S->stop || (!S->pending.empty() && free_slot(S) >= 0); });
        if (S->stop) break;
        const int si = free_slot(S);
        Slot& slot = S->slots[si];
        std::vector<Request*> batch;
        std::set<uint32_t> blocked;  // scenes whose next request cannot run in this batch
        uint32_t nviews = 0;
        uint64_t npix = 0;
        for (auto it = S->pending.begin(); it != S->pending.end();) {
            Request* r = *it;
            if (blocked.count(r->scene)) {  // one request per scene per batch, in order
                ++it;
                continue;
            }
            if (nviews + r->views.size() > S->cfg.max_batch_views || npix + r->pixels > kMaxTracePixels) break;
            if (S->cfg.hbm_budget && S->hbm_used + r->staging > S->cfg.hbm_budget) {
                blocked.insert(r->scene);  // waits for memory; later requests of the scene wait behind it
                ++it;
                continue;
            }
            batch.push_back(r);
            blocked.insert(r->scene);
            nviews += uint32_t(r->views.size());
            npix += r->pixels;
            S->hbm_used += r->staging;
            it = S->pending.erase(it);
        }
        if (batch.empty()) {  // nothing admissible until a batch completes
            S->cv_sched.wait_for(lk, std::chrono::milliseconds(50), [&] { return S->stop || S->generation != seen; });
            seen = S->generation;
            continue;
        }
        const Clock::time_point now = Clock::now();
        slot.busy = true;
        slot.reqs = batch;
        slot.scenes.clear();
        slot.waits.clear();
        for (Request* r : batch) {
            Scene* sc = S->scenes.at(r->scene);
            // the slot of the scene's latest batch in flight cannot be reused before this batch is issued (the
            // scheduler issues batches in turn), so its event still marks that batch
            slot.waits.push_back(sc->inflight && sc->last_slot >= 0 ? S->slots[sc->last_slot].done : nullptr);
            sc->inflight += 1;
            sc->last_slot = si;
            slot.scenes.push_back(sc);
        }
        slot.batch = S->next_batch++;
        for (Request* r : batch) r->admitted = true, r->t_admit = now, r->batch = slot.batch;
        for (Request* r : batch)
            if (r->flags & F184GI_REQ_INJECT_WORKER_EXIT) return;  // test hook: the worker is lost between stages
        lk.unlock();
        int rc = issue_batch(S, slot);
        lk.lock();
        if (rc) {
            const Clock::time_point t = Clock::now();
            cudaStreamSynchronize(slot.stream);
            for (size_t k = 0; k < slot.reqs.size(); ++k) {
                Request* r = slot.reqs[k];
                if (r->d_stage) cudaFree(r->d_stage), r->d_stage = nullptr;
                finish_request(S, r, slot.req_status.size() > k && slot.req_status[k] ? slot.req_status[k] : rc, t);
                slot.scenes[k]->inflight -= 1;
            }
            slot.reqs.clear();
            slot.busy = false;
            S->generation++;
            S->cv_done.notify_all();
            continue;
        }
        S->launched.push_back(si);
        S->cv_done.notify_all();
    }
}

void completer(f184gi_server* S) {
    cudaSetDevice(S->cfg.device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        S->cv_done.wait(lk, [&] { return !S->launched.empty() || S->stop; });
        if (S->launched.empty()) {
            if (S->stop) break;
            continue;
        }
        const int si = S->launched.front();
        Slot& slot = S->slots[si];
        lk.unlock();
        cudaError_t e = cudaEventSynchronize(slot.done);
        int st = e == cudaSuccess ? F184GI_OK : cuda_fail(e, "server: batch");
        if (st == F184GI_OK) {
            // kernels flag overflow / timeout on each touched scene's context (captured in stream order)
            for (size_t k = 0; k < slot.scenes.size(); ++k) {
                int rs = ctx_status_report(slot.scenes[k]->ctx, slot.h_status[k]);
                if (rs) st = rs;
            }
        }
        lk.lock();
        S->launched.pop_front();
        const Clock::time_point now = Clock::now();
        for (size_t k = 0; k < slot.reqs.size(); ++k) {
            finish_request(S, slot.reqs[k], slot.req_status[k] ? slot.req_status[k] : st, now);
            slot.scenes[k]->inflight -= 1;
        }
        S->batches += 1;
        S->batch_views += slot.tv.size();
        slot.reqs.clear();
        slot.busy = false;
        S->generation++;
        S->cv_sched.notify_all();
        S->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

int f184gi_server_create(const f184gi_server_config* cfg, f184gi_server** out) {
    if (!out) return fail(F184GI_ERR_INVALID, "server_create: out is null");
    *out = nullptr;
    f184gi_server_config c = cfg ? *cfg : f184gi_server_config{};
    if (c.slots == 0) c.slots = 2;
    if (c.slots > 4) return fail(F184GI_ERR_INVALID, "server_create: slots must be 1..4");
    if (c.max_batch_views == 0) c.max_batch_views = 64;
    if (c.max_batch_views > 4096) return fail(F184GI_ERR_INVALID, "server_create: max_batch_views too large");
    if (c.cone.diffuse_cones == 0) f184gi_cone_params_default(&c.cone);
    if (c.trace_variant > kTraceVariantCount)
        return fail(F184GI_ERR_INVALID, "server_create: trace_variant must be 0 (tune) or 1.." +
                                            std::to_string(kTraceVariantCount));
    cudaError_t e = cudaSetDevice(c.device);
    if (e != cudaSuccess) return cuda_fail(e, "server_create: device");
    f184gi_server* S = new f184gi_server();
    S->cfg = c;
    S->tc.p = c.cone;
    const double tilt = double(c.cone.diffuse_tilt_deg) * M_PI / 180.0;
    S->tc.cos_tilt = float(std::cos(tilt));
    S->tc.sin_tilt = float(std::sin(tilt));
    S->tc.tmax = 0.0f;  // per view
    trace_consts_schedule(S->tc);
    if (c.trace_variant) S->variant = int(c.trace_variant) - 1;
    S->slots.resize(c.slots);
    for (Slot& sl : S->slots) {
        if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaHostAlloc(reinterpret_cast<void**>(&sl.h_status), size_t(c.max_batch_views) * 4,
                               cudaHostAllocDefault)) != cudaSuccess) {
            f184gi_server_destroy(S);
            return cuda_fail(e, "server_create: streams");
        }
    }
    S->sched = std::thread(scheduler, S);
    S->completer = std::thread(completer, S);
    *out = S;
    return F184GI_OK;
}

int f184gi_server_destroy(f184gi_server* S) {
    if (!S) return fail(F184GI_ERR_INVALID, "server_destroy: null server");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_sched.notify_all();
    S->cv_done.notify_all();
    if (S->sched.joinable()) S->sched.join();
    if (S->completer.joinable()) S->completer.join();
    cudaDeviceSynchronize();
    for (Slot& sl : S->slots) {
        trace_graph_destroy(sl.graph);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.h_status) cudaFreeHost(sl.h_status);
    }
    for (auto& kv : S->scenes) {
        Scene* sc = kv.second;
        cudaFree(sc->d_tri);
        cudaFree(sc->d_alb);
        cudaFree(sc->d_dirty);
        cudaFreeHost(sc->h_dirty);
        if (sc->dirty_copied) cudaEventDestroy(sc->dirty_copied);
        if (sc->ctx) f184gi_destroy(sc->ctx);
        delete sc;
    }
    for (auto& kv : S->reqs) delete kv.second;
    if (S->log) std::fclose(S->log);
    delete S;
    return F184GI_OK;
}

int f184gi_server_add_scene(f184gi_server* S, uint32_t id, const f184gi_grid_desc* desc, const float* tri,
                            const uint32_t* albedo, uint64_t ntris, const f184gi_bounds* bounds,
                            const f184gi_light* light) {
    if (!S || !desc || !tri || !albedo || !bounds || !light || ntris == 0)
        return fail(F184GI_ERR_INVALID, "server_add_scene: null argument");
    for (uint64_t i = 0; i < ntris * 9; ++i)
        if (!std::isfinite(tri[i]))
            return fail(F184GI_ERR_INVALID, "server_add_scene: triangle " + std::to_string(i / 9) +
                                                " has a NaN or infinite coordinate");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->scenes.count(id)) return fail(F184GI_ERR_INVALID, "server_add_scene: scene id already registered");
        if ((S->fmt >= 0 && S->fmt != int(desc->format)) || (S->aniso >= 0 && S->aniso != int(desc->anisotropic)))
            return fail(F184GI_ERR_INVALID, "server_add_scene: all scenes of a server share format and anisotropy");
    }
    f184gi_grid_desc d = *desc;
    d.flags |= F184GI_GRID_RESIDENT_WEIGHTS;
    uint64_t need = 0;
    int rc = f184gi_grid_bytes(&d, &need);
    if (rc) return rc;
    need += ntris * 40 + voxelize_scratch_bytes(ntris, d.dim) + raster_scratch_bytes(ntris, d.shadow_res, d.shadow_res);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->cfg.hbm_budget && S->hbm_used + need > S->cfg.hbm_budget)
            return fail(F184GI_ERR_BUDGET, "server_add_scene: the scene does not fit the HBM budget");
        S->hbm_used += need;  // reserved while building
    }
    Scene* sc = new Scene();
    sc->id = id;
    sc->desc = d;
    sc->ntris = ntris;
    sc->bounds = *bounds;
    sc->light = *light;
    f184gi_config cc{S->cfg.device, 0u, 0u};
    cudaError_t e = cudaSuccess;
    if (!(rc = f184gi_create(&cc, &sc->ctx))) rc = f184gi_grid_create(sc->ctx, &d, &sc->grid);
    sc->nbricks = (d.dim / 8) * (d.dim / 8) * (d.dim / 8);
    if (!rc && ((e = cudaMalloc(&sc->d_tri, ntris * 36)) != cudaSuccess || (e = cudaMalloc(&sc->d_alb, ntris * 4)) != cudaSuccess ||
                (e = cudaMalloc(&sc->d_dirty, size_t(sc->nbricks) * 4)) != cudaSuccess ||
                (e = cudaHostAlloc(&sc->h_dirty, size_t(sc->nbricks) * 4, cudaHostAllocDefault)) != cudaSuccess ||
                (e = cudaEventCreateWithFlags(&sc->dirty_copied, cudaEventDisableTiming)) != cudaSuccess))
        rc = cuda_fail(e, "server_add_scene: allocation");
    if (!rc) {
        sc->h_tri.assign(tri, tri + ntris * 9);
        sc->flag.assign(sc->nbricks, 0);
        cudaMemcpy(sc->d_tri, tri, ntris * 36, cudaMemcpyHostToDevice);
        cudaMemcpy(sc->d_alb, albedo, ntris * 4, cudaMemcpyHostToDevice);
        rc = f184gi_voxelize(sc->ctx, sc->grid, sc->d_tri, sc->d_alb, ntris, bounds, light, nullptr, 0, nullptr);
    }
    if (!rc) rc = f184gi_mip(sc->ctx, sc->grid, 0, d.anisotropic, nullptr);
    if (!rc) rc = f184gi_sync(sc->ctx, nullptr);
    if (!rc) rc = compute_frame(*bounds, d.dim, light->direction, &sc->frame);
    if (!rc) rc = grid_internal(sc->ctx, sc->grid, &sc->chain, &sc->d_frame);
    std::lock_guard<std::mutex> lk(S->mu);
    if (rc) {
        S->hbm_used -= need;
        cudaFree(sc->d_tri);
        cudaFree(sc->d_alb);
        cudaFree(sc->d_dirty);
        cudaFreeHost(sc->h_dirty);
        if (sc->dirty_copied) cudaEventDestroy(sc->dirty_copied);
        if (sc->ctx) f184gi_destroy(sc->ctx);
        delete sc;
        return rc;
    }
    sc->bytes = need;
    S->fmt = int(d.format);
    S->aniso = int(d.anisotropic);
    S->scenes[id] = sc;
    return F184GI_OK;
}

}  // extern "C"

namespace {

// A request checked against its own fields (no server state): the copy that the server queues.
int make_request(const f184gi_request* req, Request** out) {
    *out = nullptr;
    if (req->nviews == 0 || !req->views) return fail(F184GI_ERR_INVALID, "server_submit: a request needs views");
    if (req->nmoves && !req->moves) return fail(F184GI_ERR_INVALID, "server_submit: null moves");
    for (uint32_t i = 0; i < req->nviews; ++i) {
        const f184gi_view& v = req->views[i];
        if (!v.depth || !v.normal || !v.roughness || !v.out || v.width == 0 || v.height == 0 ||
            v.width > kMaxViewSide || v.height > kMaxViewSide ||
            (v.out_format != F184GI_FMT_F32 && v.out_format != F184GI_FMT_F16))
            return fail(F184GI_ERR_INVALID, "server_submit: malformed view " + std::to_string(i));
    }
    Request* r = new Request();
    r->scene = req->scene_id;
    r->flags = req->flags;
    r->moves.assign(req->moves, req->moves + req->nmoves);
    r->views.assign(req->views, req->views + req->nviews);
    for (const f184gi_view& v : r->views) r->pixels += uint64_t(v.width) * v.height;
    r->staging = staging_bytes(*req);
    *out = r;
    return F184GI_OK;
}

// Checks against the server's scenes and limits (S->mu held).
int admit_check(f184gi_server* S, const Request* r) {
    auto it = S->scenes.find(r->scene);
    if (it == S->scenes.end()) return fail(F184GI_ERR_NOTFOUND, "server_submit: unknown scene");
    for (const f184gi_move& m : r->moves)
        if (uint64_t(m.first) + m.count > it->second->ntris)
            return fail(F184GI_ERR_INVALID, "server_submit: move range out of bounds");
    if (r->views.size() > S->cfg.max_batch_views)
        return fail(F184GI_ERR_INVALID, "server_submit: more views than max_batch_views");
    if (r->pixels > kMaxTracePixels) return fail(F184GI_ERR_INVALID, "server_submit: more than 2^36 pixels");
    if (S->cfg.hbm_budget && r->staging > S->cfg.hbm_budget)
        return fail(F184GI_ERR_BUDGET, "server_submit: the request's staging exceeds the HBM budget");
    return F184GI_OK;
}

void enqueue(f184gi_server* S, Request* r, Clock::time_point now) {
    r->ticket = S->next_ticket++;
    r->t_submit = now;
    S->reqs[r->ticket] = r;
    S->pending.push_back(r);
}

}  // namespace

extern "C" {

int f184gi_server_submit(f184gi_server* S, const f184gi_request* req, uint64_t* ticket) {
    return f184gi_server_submit_batch(S, req, 1, ticket);
}

int f184gi_server_submit_batch(f184gi_server* S, const f184gi_request* reqs, uint32_t n, uint64_t* tickets) {
    if (!S || !reqs || !tickets) return fail(F184GI_ERR_INVALID, "server_submit: null argument");
    std::vector<Request*> rs;
    rs.reserve(n);
    for (uint32_t k = 0; k < n; ++k) {
        Request* r = nullptr;
        int rc = make_request(&reqs[k], &r);
        if (rc) {
            for (Request* q : rs) delete q;
            return rc;
        }
        rs.push_back(r);
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->worker_lost) {
        for (Request* q : rs) delete q;
        return fail(F184GI_ERR_WORKER, "server_submit: the server's scheduler thread has stopped");
    }
    for (Request* r : rs) {
        int rc = admit_check(S, r);
        if (rc) {
            for (Request* q : rs) delete q;
            return rc;
        }
    }
    const Clock::time_point now = Clock::now();
    for (uint32_t k = 0; k < n; ++k) {
        enqueue(S, rs[k], now);
        tickets[k] = rs[k]->ticket;
    }
    S->cv_sched.notify_all();
    return F184GI_OK;
}

int f184gi_server_wait(f184gi_server* S, uint64_t ticket, uint32_t timeout_ms, f184gi_request_result* out) {
    if (!S) return fail(F184GI_ERR_INVALID, "server_wait: null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(F184GI_ERR_NOTFOUND, "server_wait: unknown ticket");
    Request* r = it->second;
    if (timeout_ms) {
        if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; }))
            return fail(F184GI_ERR_TIMEOUT, "server_wait: timed out");
    } else {
        S->cv_done.wait(lk, [&] { return r->done; });
    }
    if (out) {
        out->status = r->status;
        out->batch = r->batch;
        out->queued_ms = r->admitted ? ms_between(r->t_submit, r->t_admit) : 0.0;
        out->latency_ms = ms_between(r->t_submit, r->t_done);
        out->pixels = r->pixels;
    }
    return r->status == F184GI_ERR_CANCELLED ? F184GI_OK : (r->status ? fail(r->status, "server: request failed") : F184GI_OK);
}

int f184gi_server_cancel(f184gi_server* S, uint64_t ticket) {
    if (!S) return fail(F184GI_ERR_INVALID, "server_cancel: null server");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(F184GI_ERR_NOTFOUND, "server_cancel: unknown ticket");
    Request* r = it->second;
    auto p = std::find(S->pending.begin(), S->pending.end(), r);
    if (p == S->pending.end()) return fail(F184GI_ERR_INVALID, "server_cancel: the request is running or done");
    S->pending.erase(p);
    r->status = F184GI_ERR_CANCELLED;
    r->done = true;
    r->t_done = Clock::now();
    S->cancelled += 1;
    S->cv_done.notify_all();
    S->cv_sched.notify_all();
    return F184GI_OK;
}

int f184gi_server_set_log(f184gi_server* S, const char* path) {
    if (!S) return fail(F184GI_ERR_INVALID, "server_set_log: null server");
    FILE* f = nullptr;
    if (path && !(f = std::fopen(path, "a"))) return fail(F184GI_ERR_INVALID, std::string("server_set_log: cannot open ") + path);
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->log) std::fclose(S->log);
    S->log = f;
    return F184GI_OK;
}

int f184gi_server_get_stats(f184gi_server* S, f184gi_server_stats* out) {
    if (!S || !out) return fail(F184GI_ERR_INVALID, "server_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    *out = f184gi_server_stats{};
    out->requests_done = S->done_n;
    out->requests_cancelled = S->cancelled;
    out->batches = S->batches;
    out->pixels = S->pixels;
    if (!S->lat.empty()) {
        std::vector<double> l = S->lat;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) { return l[std::min(l.size() - 1, size_t(q * double(l.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double s = 0.0;
        for (double x : l) s += x;
        out->mean_ms = s / double(l.size());
    }
    out->mean_batch_views = S->batches ? double(S->batch_views) / double(S->batches) : 0.0;
    out->hbm_used = S->hbm_used;
    out->hbm_budget = S->cfg.hbm_budget;
    out->pending = uint32_t(S->pending.size());
    uint32_t inflight = 0;
    for (const Slot& sl : S->slots) inflight += sl.busy ? 1u : 0u;
    out->inflight = inflight;
    out->trace_variants = kTraceVariantCount;
    if (S->variant >= 0 && S->fmt >= 0) {
        const TraceVariant& v = kTraceVariants[S->variant];
        out->trace_variant = uint32_t(S->variant);
        out->trace_tile[0] = v.tw;
        out->trace_tile[1] = v.th;
        out->trace_ctas_per_sm = trace_persistent_blocks(uint32_t(S->fmt), S->aniso != 0, uint32_t(S->variant),
                                                         S->cfg.blocks_per_sm) /
                                 std::max(1u, sm_count());
        for (uint32_t k = 0; k < kTraceVariantCount && k < 8; ++k) out->tune_ms[k] = S->tune_ms[k];
    }
    return F184GI_OK;
}

}  // extern "C"
