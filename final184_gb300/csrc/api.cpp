// api.cpp -- the f184gi C ABI: contexts, resident grids, the three passes and inspection.
//
// A context owns device memory under an optional HBM budget: resident grids (mip chain + shadow map + frame)
// and per-pass scratch that grows on demand and is reused.  Calls are stream-ordered on the caller's stream;
// kernels report overflow/timeout through a device status word that f184gi_sync and the inspection calls read.
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "frame.h"
#include "gi_internal.h"
#include "util.cuh"

namespace f184 {

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
}  // namespace

void note_launches(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return F184GI_OK;
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? F184GI_ERR_OOM : F184GI_ERR_CUDA;
}

bool invert4(const double* m, double* inv) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? m[r * 4 + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(a[p][k], a[c][k]);
        double iv = 1.0 / a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] *= iv;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[r * 4 + c] = a[r][c + 4];
    return true;
}

int compute_frame(const f184gi_bounds& b, uint32_t dim, const float light_dir[3], f184gi_grid_frame* out) {
    std::memset(out, 0, sizeof(*out));
    const float mn[3] = {b.min.x, b.min.y, b.min.z}, mx[3] = {b.max.x, b.max.y, b.max.z};
    frame_from_bounds(mn, mx, dim, light_dir, out);
    return F184GI_OK;
}

// The frame and its FP32 pairs as the device's frame kernel writes them (same FP64 operations, no contraction in
// this file; the pairs are conversions and one subtraction per axis).
int compute_frame_block(const f184gi_bounds& b, uint32_t dim, const float light_dir[3], FrameBlock* out) {
    std::memset(out, 0, sizeof(*out));
    compute_frame(b, dim, light_dir, &out->frame);
    for (int a = 0; a < 3; ++a) {
        out->pairs.org_h[a] = float(out->frame.origin[a]);
        out->pairs.org_l[a] = float(out->frame.origin[a] - double(out->pairs.org_h[a]));
    }
    const double ivs = out->frame.inv_voxel_fixed * (1.0 / 256.0);
    out->pairs.ivs_h = float(ivs);
    out->pairs.ivs_l = float(ivs - double(out->pairs.ivs_h));
    return F184GI_OK;
}

// The diffuse cones' march recurrence, step by step as the kernel's cone loop advances it: diameter
// max(1, 2 tan (t + tl)) with the low part's product rounded first, step = step_factor * diameter and the
// error-free sum t + step (this file is compiled without floating-point contraction).
void trace_consts_schedule(TraceConsts& tc) {
    float t = tc.p.start_offset, tl = 0.0f;
    const float d2 = 2.0f * tc.p.diffuse_tan_half;
    for (uint32_t k = 0; k < kDiffuseSched; ++k) {
        const float diam = std::max(1.0f, std::fma(d2, t, d2 * tl));
        tc.sched[k] = SchedEntry{t, tl, diam, std::max(std::log2(diam), 0.0f)};
        const float step = tc.p.step_factor * diam;
        const float ts = t + step, tb = ts - t;
        tl = tl + ((t - (ts - tb)) + (step - tb));
        t = ts;
    }
}

}  // namespace f184

using namespace f184;

struct GridObj {
    f184gi_grid_desc desc{};
    ChainLayout chain{};
    size_t chain_bytes = 0;
    unsigned long long* shadow = nullptr;
    size_t shadow_bytes = 0;
    uint32_t* counts = nullptr;
    size_t counts_bytes = 0;
    float4* weights = nullptr;  // resident mean injection weights (F184GI_GRID_RESIDENT_WEIGHTS)
    size_t weights_bytes = 0;
    f184gi_grid_frame* d_frame = nullptr;
    bool voxelized = false;
    // levels 1 .. min(3, levels - 1) agree with L0: written with it by the last voxelizations (isotropic FP32
    // grids), or by a full mip build since; a pointer handed out by f184gi_grid_level_ptr clears it
    bool low_levels_current = false;
    f184gi_light light{};  // the light of the last voxelization (the march shades with it)
};

struct f184gi_ctx {
    int device = 0;
    uint64_t budget = 0;
    uint64_t used = 0;
    std::map<uint32_t, GridObj> grids;
    uint32_t next_id = 1;
    Scratch raster, vox, trace, misc, keys, counts;
    uint32_t* d_status = nullptr;
    bool failed = false;  // a bulk-copy wait expired (kStatusCopyTimeout): every later call is refused
    TraceStaging* trace_stage = nullptr;
    // voxelize forks the triangle lists onto aux (after the frame) beside the shadow raster on the caller's
    // stream, and joins before the bricks
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace {

int dev_alloc(f184gi_ctx* c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return F184GI_OK;
    if (c->budget && c->used + bytes > c->budget)
        return fail(F184GI_ERR_BUDGET, "allocation of " + std::to_string(bytes) + " bytes exceeds the HBM budget");
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(F184GI_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c->used += bytes;
    return F184GI_OK;
}

void dev_free(f184gi_ctx* c, void* p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    c->used -= bytes;
}

// Grow a scratch slot to at least `bytes` (contents are not preserved).
int scratch_get(f184gi_ctx* c, Scratch& s, size_t bytes) {
    if (s.bytes >= bytes) return F184GI_OK;
    if (s.ptr) {
        cudaError_t e = cudaDeviceSynchronize();  // the old buffer may still be in use by queued work
        if (e != cudaSuccess) return cuda_fail(e, "scratch resize");
        dev_free(c, s.ptr, s.bytes);
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = bytes + bytes / 8;
    int rc = dev_alloc(c, &s.ptr, want);
    if (rc) return rc;
    s.bytes = want;
    return F184GI_OK;
}

bool pow2(uint32_t x) { return x && !(x & (x - 1)); }

int check_desc(const f184gi_grid_desc* d) {
    if (!d) return fail(F184GI_ERR_INVALID, "grid descriptor is null");
    if (!pow2(d->dim) || d->dim < 16 || d->dim > 512) return fail(F184GI_ERR_INVALID, "grid dim must be a power of two in 16..512");
    uint32_t maxl = 0;
    for (uint32_t x = d->dim; x > 1; x >>= 1) ++maxl;  // log2(dim): keeps a 2^3 top level
    if (d->levels < 1 || d->levels > maxl || d->levels > uint32_t(kMaxLevels))
        return fail(F184GI_ERR_INVALID, "grid levels must be in 1..log2(dim)");
    if (d->format != F184GI_FMT_F32 && d->format != F184GI_FMT_F16 && d->format != F184GI_FMT_RG16)
        return fail(F184GI_ERR_INVALID, "unknown grid format");
    if (d->format == F184GI_FMT_RG16 && (d->levels != 1 || d->anisotropic || d->flags))
        return fail(F184GI_ERR_INVALID, "an RG16 (reference) grid has one level, no anisotropy and no flags");
    if (d->shadow_res < 64 || d->shadow_res > 8192) return fail(F184GI_ERR_INVALID, "shadow_res must be in 64..8192");
    if (d->anisotropic > 1) return fail(F184GI_ERR_INVALID, "anisotropic must be 0 or 1");
    return F184GI_OK;
}

uint32_t format_bytes(uint32_t format) {
    return format == F184GI_FMT_F32 ? 16u : (format == F184GI_FMT_F16 ? 8u : 4u);
}

ChainLayout layout_for(const f184gi_grid_desc& d, void* base) {
    ChainLayout c{};
    c.base = base;
    c.dim = d.dim;
    c.levels = d.levels;
    c.format = d.format;
    c.aniso = d.anisotropic;
    c.esz = format_bytes(d.format);
    uint64_t off = 0;
    for (uint32_t l = 0; l < d.levels; ++l) {
        uint64_t dl = d.dim >> l;
        c.ldim[l] = uint32_t(dl);
        c.off[l] = off;
        c.vol[l] = l == 0 ? dl * dl * dl : (dl + 2) * (dl + 2) * (dl + 2);  // levels >= 1: a ring of zeros
        off += c.vol[l] * ((d.anisotropic && l > 0) ? 6 : 1);
    }
    return c;
}

uint64_t chain_elems(const f184gi_grid_desc& d) {
    ChainLayout c = layout_for(d, nullptr);
    uint32_t l = d.levels - 1;
    return c.off[l] + c.vol[l] * ((d.anisotropic && l > 0) ? 6 : 1);
}

// A context whose bulk-copy wait expired refuses further work (kStatusCopyTimeout).
int refused(const f184gi_ctx* c, const char* what) {
    return c->failed ? fail(F184GI_ERR_TIMEOUT, std::string(what) + ": the context failed (a bounded wait on a bulk "
                                                                      "copy expired); create a new one")
                     : F184GI_OK;
}

GridObj* find_grid(f184gi_ctx* c, uint32_t id) {
    auto it = c->grids.find(id);
    return it == c->grids.end() ? nullptr : &it->second;
}

int decode_status(f184gi_ctx* c, uint32_t st) {
    if (!st) return F184GI_OK;
    if (st & kStatusCopyTimeout) {
        c->failed = true;
        return fail(F184GI_ERR_TIMEOUT, "a bounded wait on a bulk copy expired; the copy may still be in flight, so the "
                                        "context refuses further calls");
    }
    if (st & kStatusTimeout) return fail(F184GI_ERR_TIMEOUT, "a bounded device wait expired");
    if (st & kStatusOverflow) return fail(F184GI_ERR_OVERFLOW, "a bounded device structure overflowed");
    if (st & kStatusNonFinite)
        return fail(F184GI_ERR_INVALID, "triangles with a NaN or infinite coordinate were skipped");
    return fail(F184GI_ERR_INVALID, "geometry outside the fixed-point range was skipped");
}

int read_status(f184gi_ctx* c) {
    uint32_t st = 0;
    cudaError_t e = cudaMemcpy(&st, c->d_status, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (!st) return F184GI_OK;
    cudaMemset(c->d_status, 0, 4);
    return decode_status(c, st);
}

}  // namespace

namespace {
// NVTX range over one pass of the C ABI (host-side issue of its kernels), for Nsight timelines
struct PassRange {
    explicit PassRange(const char* name) { nvtxRangePushA(name); }
    ~PassRange() { nvtxRangePop(); }
};
}  // namespace

extern "C" {

const char* f184gi_last_error(void) { return g_last_error.c_str(); }
uint64_t f184gi_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }
int f184gi_abi_version(void) { return F184GI_ABI_VERSION; }

int f184gi_create(const f184gi_config* cfg, f184gi_ctx** out) {
    if (!out) return fail(F184GI_ERR_INVALID, "create: out is null");
    *out = nullptr;
    int device = cfg ? cfg->device : 0;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    f184gi_ctx* c = new f184gi_ctx();
    c->device = device;
    c->budget = cfg ? cfg->hbm_budget : 0;
    void* st = nullptr;
    int rc = dev_alloc(c, &st, 256);
    if (rc) {
        delete c;
        return rc;
    }
    c->d_status = static_cast<uint32_t*>(st);
    cudaMemset(c->d_status, 0, 4);
    // The lists chain is a run of short latency-bound kernels: at the highest stream priority its blocks are
    // scheduled ahead of another request's trace when two requests overlap on the device (two request lanes:
    // 2.35 -> 2.29 ms per plain-large request; one lane unchanged).
    int least_prio = 0, greatest_prio = 0;
    cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio);
    if ((e = cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, greatest_prio)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming)) != cudaSuccess) {
        f184gi_destroy(c);
        return cuda_fail(e, "create: auxiliary stream");
    }
    *out = c;
    return F184GI_OK;
}

int f184gi_destroy(f184gi_ctx* c) {
    if (!c) return fail(F184GI_ERR_INVALID, "destroy: null context");
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (auto& kv : c->grids) {
        GridObj& g = kv.second;
        dev_free(c, g.chain.base, g.chain_bytes);
        dev_free(c, g.shadow, g.shadow_bytes);
        dev_free(c, g.counts, g.counts_bytes);
        dev_free(c, g.weights, g.weights_bytes);
        dev_free(c, g.d_frame, kFrameAllocBytes);
    }
    for (Scratch* s : {&c->raster, &c->vox, &c->trace, &c->misc, &c->keys, &c->counts}) dev_free(c, s->ptr, s->bytes);
    trace_staging_destroy(c->trace_stage);
    dev_free(c, c->d_status, 256);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->aux) cudaStreamDestroy(c->aux);
    delete c;
    return F184GI_OK;
}

int f184gi_memory_used(f184gi_ctx* c, uint64_t* bytes) {
    if (!c || !bytes) return fail(F184GI_ERR_INVALID, "memory_used: null argument");
    *bytes = c->used;
    return F184GI_OK;
}

int f184gi_grid_bytes(const f184gi_grid_desc* d, uint64_t* bytes) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!bytes) return fail(F184GI_ERR_INVALID, "grid_bytes: null output");
    uint64_t esz = format_bytes(d->format);
    uint64_t b = chain_elems(*d) * esz + uint64_t(d->shadow_res) * d->shadow_res * 8 + kFrameAllocBytes;
    if (d->flags & F184GI_GRID_KEEP_COUNTS) b += uint64_t(d->dim) * d->dim * d->dim * 4;
    if (d->flags & F184GI_GRID_RESIDENT_WEIGHTS) b += uint64_t(d->dim) * d->dim * d->dim * 16;
    *bytes = b;
    return F184GI_OK;
}

int f184gi_grid_create(f184gi_ctx* c, const f184gi_grid_desc* d, uint32_t* grid) {
    if (!c || !grid) return fail(F184GI_ERR_INVALID, "grid_create: null argument");
    int rc = check_desc(d);
    if (rc) return rc;
    GridObj g;
    g.desc = *d;
    uint64_t esz = format_bytes(d->format);
    g.chain_bytes = chain_elems(*d) * esz;
    void* base = nullptr;
    if ((rc = dev_alloc(c, &base, g.chain_bytes))) return rc;
    cudaMemset(base, 0, g.chain_bytes);  // the zero rings of levels >= 1 are never written again
    g.chain = layout_for(*d, base);
    g.shadow_bytes = size_t(d->shadow_res) * d->shadow_res * 8;
    void* sh = nullptr;
    if ((rc = dev_alloc(c, &sh, g.shadow_bytes))) {
        dev_free(c, base, g.chain_bytes);
        return rc;
    }
    g.shadow = static_cast<unsigned long long*>(sh);
    void* fr = nullptr;
    if ((rc = dev_alloc(c, &fr, kFrameAllocBytes))) {
        dev_free(c, base, g.chain_bytes);
        dev_free(c, sh, g.shadow_bytes);
        return rc;
    }
    g.d_frame = static_cast<f184gi_grid_frame*>(fr);
    if (d->flags & F184GI_GRID_KEEP_COUNTS) {
        g.counts_bytes = size_t(d->dim) * d->dim * d->dim * 4;
        void* cp = nullptr;
        if ((rc = dev_alloc(c, &cp, g.counts_bytes))) {
            dev_free(c, base, g.chain_bytes);
            dev_free(c, sh, g.shadow_bytes);
            dev_free(c, fr, kFrameAllocBytes);
            return rc;
        }
        g.counts = static_cast<uint32_t*>(cp);
        cudaMemset(g.counts, 0, g.counts_bytes);
    }
    if (d->flags & F184GI_GRID_RESIDENT_WEIGHTS) {
        g.weights_bytes = size_t(d->dim) * d->dim * d->dim * 16;
        void* wp = nullptr;
        if ((rc = dev_alloc(c, &wp, g.weights_bytes))) {
            dev_free(c, base, g.chain_bytes);
            dev_free(c, sh, g.shadow_bytes);
            dev_free(c, fr, kFrameAllocBytes);
            dev_free(c, g.counts, g.counts_bytes);
            return rc;
        }
        g.weights = static_cast<float4*>(wp);
        cudaMemset(g.weights, 0, g.weights_bytes);
    }
    cudaMemset(base, 0, g.chain_bytes);
    cudaMemset(fr, 0, kFrameAllocBytes);
    uint32_t id = c->next_id++;
    c->grids[id] = g;
    *grid = id;
    return F184GI_OK;
}

int f184gi_grid_destroy(f184gi_ctx* c, uint32_t grid) {
    if (!c) return fail(F184GI_ERR_INVALID, "grid_destroy: null context");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_destroy: unknown grid");
    cudaDeviceSynchronize();
    dev_free(c, g->chain.base, g->chain_bytes);
    dev_free(c, g->shadow, g->shadow_bytes);
    dev_free(c, g->counts, g->counts_bytes);
    dev_free(c, g->weights, g->weights_bytes);
    dev_free(c, g->d_frame, kFrameAllocBytes);
    c->grids.erase(grid);
    return F184GI_OK;
}

int f184gi_voxelize(f184gi_ctx* c, uint32_t grid, const float* tri, const uint32_t* albedo, uint64_t ntris,
                    const f184gi_bounds* bounds, const f184gi_light* light, const uint32_t* dirty, uint32_t ndirty,
                    void* stream) {
    PassRange range("f184gi_voxelize");
    if (!c || !light) return fail(F184GI_ERR_INVALID, "voxelize: null argument");
    if (int rc0 = refused(c, "voxelize")) return rc0;
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "voxelize: unknown grid");
    if (ntris && (!tri || !albedo)) return fail(F184GI_ERR_INVALID, "voxelize: null triangle buffers");
    if (ndirty && !dirty) return fail(F184GI_ERR_INVALID, "voxelize: null dirty list");
    if (!bounds && ntris == 0) return fail(F184GI_ERR_INVALID, "voxelize: no triangles and no bounds");
    float ld = light->direction[0] * light->direction[0] + light->direction[1] * light->direction[1] +
               light->direction[2] * light->direction[2];
    if (!(ld > 0.0f) || !std::isfinite(ld)) return fail(F184GI_ERR_INVALID, "voxelize: light direction is zero");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const f184gi_grid_desc& d = g->desc;
    int rc = scratch_get(c, c->misc, 4096);
    if (rc) return rc;
    if (d.format == F184GI_FMT_RG16 && ndirty)
        return fail(F184GI_ERR_INVALID, "voxelize: an RG16 grid is always voxelized whole");
    if (g->weights && ndirty && !g->voxelized)
        return fail(F184GI_ERR_INVALID, "voxelize: a dirty-brick update needs one full voxelization first");
    if ((rc = scratch_get(c, c->raster, raster_scratch_bytes(ntris, d.shadow_res, d.shadow_res)))) return rc;
    if ((rc = scratch_get(c, c->vox, d.format == F184GI_FMT_RG16 ? refvox_scratch_bytes(ntris, d.dim)
                                                                   : voxelize_scratch_bytes(ntris, d.dim))))
        return rc;
    if ((rc = frame_launch(tri, ntris, bounds, d.dim, light->direction, g->d_frame, c->misc.ptr, s))) return rc;
    VoxelizeJob vj{};
    vj.tri = tri;
    vj.albedo = albedo;
    vj.ntris = ntris;
    vj.d_frame = g->d_frame;
    vj.light = *light;
    vj.chain = g->chain;
    vj.shadow_keys = g->shadow;
    vj.shadow_res = d.shadow_res;
    vj.counts = g->counts;
    vj.dirty_bricks = dirty;
    vj.ndirty = ndirty;
    vj.weights = g->weights;
    // isotropic FP32 grids written directly (no resident weights): each brick CTA also writes its block of levels
    // 1..3, so f184gi_mip continues from level 3 instead of re-reading L0.  A dirty-brick update rewrites only its
    // bricks' blocks, so the others must already agree with L0.
    const bool fuse = d.format == F184GI_FMT_F32 && !d.anisotropic && !g->weights;
    vj.mip_levels = fuse && (!ndirty || g->low_levels_current) ? std::min(3u, d.levels - 1) : 0u;
    const bool lists = d.format != F184GI_FMT_RG16;
    cudaError_t e;
    if (lists) {  // the triangle lists need the frame, not the shadow map: build them beside the raster
        if ((e = cudaEventRecord(c->ev_fork, s)) != cudaSuccess || (e = cudaStreamWaitEvent(c->aux, c->ev_fork, 0)) != cudaSuccess)
            return cuda_fail(e, "voxelize: fork");
        if ((rc = voxelize_lists_launch(vj, c->vox.ptr, c->vox.bytes, c->d_status, c->aux))) return rc;
        // with resident weights the bricks write the geometry-only mean weights: no shadow map needed either
        if (g->weights && (rc = voxelize_bricks_launch(vj, c->vox.ptr, c->vox.bytes, c->d_status, c->aux)))
            return rc;
        if ((e = cudaEventRecord(c->ev_join, c->aux)) != cudaSuccess) return cuda_fail(e, "voxelize: join");
    }
    // shadow map over the grid's light frame
    RasterJob rj{};
    rj.tri = tri;
    rj.ntris = ntris;
    rj.d_M = g->d_frame->light_clip;
    rj.width = rj.height = d.shadow_res;
    rj.keys = g->shadow;
    rc = raster_launch(rj, c->raster.ptr, c->raster.bytes, c->d_status, s);
    if (lists && (e = cudaStreamWaitEvent(s, c->ev_join, 0)) != cudaSuccess) return cuda_fail(e, "voxelize: join");
    if (rc) return rc;
    g->light = *light;
    if (d.format == F184GI_FMT_RG16) {  // the reference's volume: 565 albedo and normal of the last fragment
        if ((rc = refvox_launch(tri, albedo, ntris, g->d_frame, d.dim, static_cast<uint32_t*>(g->chain.base),
                                c->vox.ptr, c->vox.bytes, c->d_status, s)))
            return rc;
        g->voxelized = true;
        return F184GI_OK;
    }
    g->low_levels_current = false;
    if (!g->weights && (rc = voxelize_bricks_launch(vj, c->vox.ptr, c->vox.bytes, c->d_status, s))) return rc;
    if (g->weights && (rc = relight_launch(g->weights, g->d_frame, g->chain, *light, g->shadow, d.shadow_res, s)))
        return rc;
    g->low_levels_current = vj.mip_levels > 0;
    g->voxelized = true;
    return F184GI_OK;
}

int f184gi_apply_moves(f184gi_ctx* c, float* tri_xyz, const f184gi_move* moves, uint32_t nmoves, uint64_t ntris,
                       void* stream) {
    if (!c || (nmoves && (!moves || !tri_xyz))) return fail(F184GI_ERR_INVALID, "apply_moves: null argument");
    for (uint32_t i = 0; i < nmoves; ++i)
        if (uint64_t(moves[i].first) + moves[i].count > ntris)
            return fail(F184GI_ERR_INVALID, "apply_moves: triangle range out of bounds");
    return moves_launch(tri_xyz, moves, nmoves, static_cast<cudaStream_t>(stream));
}

int f184gi_mip(f184gi_ctx* c, uint32_t grid, uint32_t levels, uint32_t anisotropic, void* stream) {
    PassRange range("f184gi_mip");
    if (!c) return fail(F184GI_ERR_INVALID, "mip: null context");
    if (int rc0 = refused(c, "mip")) return rc0;
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "mip: unknown grid");
    if (anisotropic != g->desc.anisotropic) return fail(F184GI_ERR_INVALID, "mip: anisotropy differs from the grid's");
    if (g->desc.format == F184GI_FMT_RG16) return fail(F184GI_ERR_INVALID, "mip: an RG16 grid has one level");
    if (levels == 0 || levels > g->desc.levels) levels = g->desc.levels;
    const uint32_t low = std::min(3u, g->desc.levels - 1);
    // levels 1..low written with L0 by the voxelization: the chain continues from level `low` (the same bytes as
    // a build from L0, whose levels 1..4 come from the same 2x2x2 means of FP32 values)
    const uint32_t from = g->low_levels_current ? std::min(low, levels - 1) : 0u;
    int rc = mip_launch(g->chain, levels, from, c->d_status, static_cast<cudaStream_t>(stream));
    if (!rc && levels - 1 >= low && g->desc.format == F184GI_FMT_F32 && !g->desc.anisotropic)
        g->low_levels_current = true;
    return rc;
}

void f184gi_cone_params_default(f184gi_cone_params* p) {
    if (!p) return;
    p->diffuse_cones = 5;
    p->diffuse_tan_half = 0.57735026918962576f;
    p->diffuse_tilt_deg = 60.0f;
    p->step_factor = 0.5f;
    p->max_distance = 0.0f;
    p->alpha_stop = 1.0f;
    p->start_offset = 1.0f;
    p->min_spec_tan_half = 0.05f;
    p->specular = 1;
    p->pad = 0;
}

namespace {
// f184gi_trace; with d_counts set, through the instrumented kernel that adds its totals there
int trace_views(f184gi_ctx* c, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                const f184gi_cone_params* params, void* stream, unsigned long long* d_counts) {
    if (!c || (nviews && !views)) return fail(F184GI_ERR_INVALID, "trace: null argument");
    if (int rc0 = refused(c, "trace")) return rc0;
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "trace: unknown grid");
    if (g->desc.format == F184GI_FMT_RG16) return fail(F184GI_ERR_INVALID, "trace: an RG16 grid is marched (f184gi_march)");
    TraceConsts tc{};
    if (params)
        tc.p = *params;
    else
        f184gi_cone_params_default(&tc.p);
    // bounded marches: a cone advances at least step_factor/2 voxels per sample over at most max_distance
    if (!(tc.p.step_factor >= 0.05f && tc.p.step_factor <= 4.0f) || !(tc.p.diffuse_tan_half > 0.0f) ||
        !(tc.p.diffuse_tan_half <= 8.0f) || !(tc.p.min_spec_tan_half > 0.0f) || !(tc.p.start_offset >= 0.0f) ||
        !(tc.p.start_offset <= 64.0f) || !(tc.p.max_distance <= 1.0e5f) || !(tc.p.alpha_stop > 0.0f) ||
        !std::isfinite(tc.p.diffuse_tilt_deg) || (tc.p.diffuse_cones != 1 && tc.p.diffuse_cones != 5))
        return fail(F184GI_ERR_INVALID, "trace: cone parameters out of range");
    tc.tmax = tc.p.max_distance > 0.0f ? tc.p.max_distance : float(double(g->desc.dim) * std::sqrt(3.0));
    double tilt = double(tc.p.diffuse_tilt_deg) * M_PI / 180.0;
    tc.cos_tilt = float(std::cos(tilt));
    tc.sin_tilt = float(std::sin(tilt));
    trace_consts_schedule(tc);
    std::vector<TraceView> tv(nviews);
    uint64_t pixels = 0;
    for (uint32_t i = 0; i < nviews; ++i) {
        const f184gi_view& v = views[i];
        if (!v.depth || !v.normal || !v.roughness || !v.out || v.width == 0 || v.height == 0)
            return fail(F184GI_ERR_INVALID, "trace: view " + std::to_string(i) + " has null buffers or zero size");
        if (v.width > kMaxViewSide || v.height > kMaxViewSide)
            return fail(F184GI_ERR_INVALID, "trace: view " + std::to_string(i) + " is larger than " +
                                                std::to_string(kMaxViewSide) + " pixels on a side");
        if ((pixels += uint64_t(v.width) * v.height) > kMaxTracePixels)
            return fail(F184GI_ERR_INVALID, "trace: the views hold more than 2^36 pixels in all");
        if (v.out_format != F184GI_FMT_F32 && v.out_format != F184GI_FMT_F16)
            return fail(F184GI_ERR_INVALID, "trace: unknown output format");
        double V[16], P[16], IV[16], IP[16];
        for (int k = 0; k < 16; ++k) V[k] = v.view[k], P[k] = v.proj[k];
        if (!invert4(V, IV) || !invert4(P, IP)) return fail(F184GI_ERR_INVALID, "trace: singular view or projection");
        TraceView& t = tv[i];
        trace_view_set_inverses(t, IP, IV);
        t.eye[0] = float(IV[3]);
        t.eye[1] = float(IV[7]);
        t.eye[2] = float(IV[11]);
        t.width = v.width;
        t.height = v.height;
        t.depth = v.depth;
        t.normal = v.normal;
        t.rough = v.roughness;
        t.out = v.out;
        t.out_format = v.out_format;
    }
    int rc = scratch_get(c, c->trace, trace_scratch_bytes(nviews));
    if (rc) return rc;
    tc.counts = d_counts;
    return trace_launch(g->chain, tc, g->d_frame, tv.data(), nviews, c->trace.ptr, c->trace.bytes,
                        trace_default_variant(g->chain.format, g->chain.aniso != 0),
                        &c->trace_stage, static_cast<cudaStream_t>(stream), d_counts != nullptr);
}
}  // namespace

int f184gi_trace(f184gi_ctx* c, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                 const f184gi_cone_params* params, void* stream) {
    PassRange range("f184gi_trace");
    return trace_views(c, grid, views, nviews, params, stream, nullptr);
}

int f184gi_trace_count(f184gi_ctx* c, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                       const f184gi_cone_params* params, uint64_t counts[2], void* stream) {
    if (!c || !counts) return fail(F184GI_ERR_INVALID, "trace_count: null argument");
    int rc = scratch_get(c, c->counts, 2 * sizeof(unsigned long long));
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* d = static_cast<unsigned long long*>(c->counts.ptr);
    cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_fail(e, "trace_count: reset");
    if ((rc = trace_views(c, grid, views, nviews, params, stream, d))) return rc;
    unsigned long long h[2] = {0, 0};
    if ((e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "trace_count: totals");
    counts[0] = h[0];
    counts[1] = h[1];
    return F184GI_OK;
}

void f184gi_march_params_default(f184gi_march_params* p) {
    if (!p) return;
    *p = f184gi_march_params{};
    p->rays = 4;
    p->second_bounce = 1;
    p->max_steps = 60;
    p->frame = 0;
    p->step_size = 0.2f;
    p->normal_offset = 0.06f;
    p->shadow_bias = 0.005f;
    p->sky[0] = 0.7f;
    p->sky[1] = 0.8f;
    p->sky[2] = 1.0f;
    p->sky_scale = 0.4f;
}

int f184gi_march(f184gi_ctx* c, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                 const f184gi_march_params* params, void* stream) {
    if (!c || (nviews && !views)) return fail(F184GI_ERR_INVALID, "march: null argument");
    if (int rc0 = refused(c, "march")) return rc0;
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "march: unknown grid");
    if (g->desc.format != F184GI_FMT_RG16) return fail(F184GI_ERR_INVALID, "march: the grid is not an RG16 grid");
    if (!g->voxelized) return fail(F184GI_ERR_INVALID, "march: the grid has not been voxelized");
    MarchJobDev J{};
    if (params)
        J.p = *params;
    else
        f184gi_march_params_default(&J.p);
    if (J.p.rays < 1 || J.p.rays > 64 || J.p.max_steps > 4096 || !(J.p.step_size > 0.0f) ||
        !std::isfinite(J.p.step_size) || !std::isfinite(J.p.normal_offset) || !std::isfinite(J.p.shadow_bias))
        return fail(F184GI_ERR_INVALID, "march: parameters out of range");
    J.vol = static_cast<const uint32_t*>(g->chain.base);
    J.shadow = g->shadow;
    J.frame_ptr = g->d_frame;
    J.dim = g->desc.dim;
    J.res = g->desc.shadow_res;
    for (int a = 0; a < 3; ++a) J.lum[a] = g->light.luminance[a], J.light_dir[a] = g->light.direction[a];
    // the 565 decode, pow(k / 31, 2.2) and pow(k / 63, 2.2) of the FP32 quotients (indirect.frag:89-95,157)
    for (int k = 0; k < 32; ++k) J.pow5[k] = float(std::pow(double(float(k) / 31.0f), 2.2));
    for (int k = 0; k < 64; ++k) J.pow6[k] = float(std::pow(double(float(k) / 63.0f), 2.2));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (uint32_t i = 0; i < nviews; ++i) {
        const f184gi_view& v = views[i];
        if (!v.depth || !v.normal || !v.out || v.width == 0 || v.height == 0 || v.width > 16384 || v.height > 16384)
            return fail(F184GI_ERR_INVALID, "march: view " + std::to_string(i) + " has null buffers or a bad size");
        double V[16], P[16], IV[16], IP[16];
        for (int k = 0; k < 16; ++k) V[k] = v.view[k], P[k] = v.proj[k];
        if (!invert4(V, IV) || !invert4(P, IP)) return fail(F184GI_ERR_INVALID, "march: singular view or projection");
        MarchViewDev mv{};
        for (int k = 0; k < 16; ++k) mv.iview[k] = float(IV[k]), mv.iproj[k] = float(IP[k]);
        for (int k = 0; k < 8; ++k) mv.iproj_zw[k] = IP[8 + k];
        mv.width = v.width;
        mv.height = v.height;
        mv.depth = v.depth;
        mv.normal = v.normal;
        mv.out = v.out;
        int rc = march_launch(J, mv, s);
        if (rc) return rc;
    }
    return F184GI_OK;
}

int f184gi_blur(f184gi_ctx* c, const float* in, const float* depth, uint32_t width, uint32_t height, float* out,
                void* stream) {
    if (!c || !in || !depth || !out) return fail(F184GI_ERR_INVALID, "blur: null argument");
    if (int rc0 = refused(c, "blur")) return rc0;
    if (width == 0 || height == 0 || width > 16384 || height > 16384) return fail(F184GI_ERR_INVALID, "blur: bad size");
    if (in == out) return fail(F184GI_ERR_INVALID, "blur: the output may not alias the input");
    int rc = scratch_get(c, c->keys, size_t(width) * height * 16);
    if (rc) return rc;
    return blur_launch(in, depth, width, height, static_cast<float*>(c->keys.ptr), out, static_cast<cudaStream_t>(stream));
}

int f184gi_gbuffer(f184gi_ctx* c, const float* tri, const float* rough, uint64_t ntris, const f184gi_view* view,
                   uint32_t* tri_id_out, void* stream) {
    PassRange range("f184gi_gbuffer");
    if (!c || !view || !tri || !rough) return fail(F184GI_ERR_INVALID, "gbuffer: null argument");
    if (int rc0 = refused(c, "gbuffer")) return rc0;
    if (!view->depth || !view->normal || !view->roughness) return fail(F184GI_ERR_INVALID, "gbuffer: null G-buffer planes");
    if (view->width == 0 || view->height == 0 || view->width > kMaxRasterSide || view->height > kMaxRasterSide)
        return fail(F184GI_ERR_INVALID, "gbuffer: view sides must be 1.." + std::to_string(kMaxRasterSide) + " pixels");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    RasterJob rj{};
    rj.tri = tri;
    rj.ntris = ntris;
    // clip = proj * view, FP64
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) {
            double acc = 0.0;
            for (int j = 0; j < 4; ++j) acc += double(view->proj[r * 4 + j]) * double(view->view[j * 4 + k]);
            rj.M[r * 4 + k] = acc;
        }
    rj.d_M = nullptr;
    rj.width = view->width;
    rj.height = view->height;
    int rc = scratch_get(c, c->keys, size_t(view->width) * view->height * 8);
    if (rc) return rc;
    rj.keys = static_cast<unsigned long long*>(c->keys.ptr);
    if ((rc = scratch_get(c, c->raster, raster_scratch_bytes(ntris, view->width, view->height)))) return rc;
    if ((rc = raster_launch(rj, c->raster.ptr, c->raster.bytes, c->d_status, s))) return rc;
    double V[16], IV[16];
    for (int k = 0; k < 16; ++k) V[k] = view->view[k];
    if (!invert4(V, IV)) return fail(F184GI_ERR_INVALID, "gbuffer: singular view matrix");
    const float eye[3] = {float(IV[3]), float(IV[7]), float(IV[11])};
    return gbuffer_resolve_launch(rj.keys, view->width, view->height, tri, rough, view->view, eye,
                                  const_cast<float*>(view->depth), const_cast<uint32_t*>(view->normal),
                                  const_cast<uint16_t*>(view->roughness), tri_id_out, s);
}

int f184gi_transform(f184gi_ctx* c, const float* obj_xyz, uint64_t ntris, const float model[12], float* world_xyz,
                     void* stream) {
    if (!c || !model || (ntris && (!obj_xyz || !world_xyz))) return fail(F184GI_ERR_INVALID, "transform: null argument");
    return transform_launch(obj_xyz, ntris, model, world_xyz, static_cast<cudaStream_t>(stream));
}

int f184gi_selftest_bounded_wait(f184gi_ctx* c, uint32_t polls, uint32_t complete, void* stream) {
    if (!c) return fail(F184GI_ERR_INVALID, "selftest_bounded_wait: null context");
    if (polls == 0 || polls > (1u << 24)) return fail(F184GI_ERR_INVALID, "selftest_bounded_wait: polls must be in 1..2^24");
    if (complete > 2) return fail(F184GI_ERR_INVALID, "selftest_bounded_wait: complete must be 0, 1 or 2");
    return bounded_wait_selftest_launch(polls, complete, c->d_status, static_cast<cudaStream_t>(stream));
}

int f184gi_sync(f184gi_ctx* c, void* stream) {
    if (!c) return fail(F184GI_ERR_INVALID, "sync: null context");
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "sync");
    return read_status(c);
}

int f184gi_frame_from_bounds(const f184gi_bounds* b, uint32_t dim, const float light_dir[3], f184gi_grid_frame* out) {
    if (!b || !light_dir || !out) return fail(F184GI_ERR_INVALID, "frame_from_bounds: null argument");
    if (dim < 4) return fail(F184GI_ERR_INVALID, "frame_from_bounds: dim too small");
    return compute_frame(*b, dim, light_dir, out);
}

int f184gi_grid_get_frame(f184gi_ctx* c, uint32_t grid, f184gi_grid_frame* out) {
    if (!c || !out) return fail(F184GI_ERR_INVALID, "grid_get_frame: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_get_frame: unknown grid");
    cudaError_t e = cudaMemcpy(out, g->d_frame, sizeof(*out), cudaMemcpyDeviceToHost);
    return cuda_fail(e, "grid_get_frame");
}

int f184gi_grid_read_level(f184gi_ctx* c, uint32_t grid, uint32_t level, uint32_t dir, float* host) {
    if (!c || !host) return fail(F184GI_ERR_INVALID, "grid_read_level: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_read_level: unknown grid");
    if (level >= g->desc.levels) return fail(F184GI_ERR_INVALID, "grid_read_level: level out of range");
    if (dir > 0 && !(g->desc.anisotropic && level > 0 && dir < 6)) return fail(F184GI_ERR_INVALID, "grid_read_level: bad direction");
    uint64_t d = g->chain.ldim[level];
    if (g->desc.format == F184GI_FMT_RG16) {  // packed uint32 per voxel, x fastest
        cudaDeviceSynchronize();
        cudaError_t e = cudaMemcpy(host, g->chain.base, size_t(d * d * d) * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "grid_read_level");
        return read_status(c);
    }
    size_t bytes = size_t(d * d * d) * 16;
    int rc = scratch_get(c, c->misc, bytes);
    if (rc) return rc;
    cudaDeviceSynchronize();
    if ((rc = read_level_launch(g->chain, level, dir, static_cast<float*>(c->misc.ptr), nullptr))) return rc;
    cudaError_t e = cudaMemcpy(host, c->misc.ptr, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "grid_read_level");
    return read_status(c);
}

int f184gi_grid_read_shadow(f184gi_ctx* c, uint32_t grid, float* host) {
    if (!c || !host) return fail(F184GI_ERR_INVALID, "grid_read_shadow: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_read_shadow: unknown grid");
    uint64_t n = uint64_t(g->desc.shadow_res) * g->desc.shadow_res;
    std::vector<unsigned long long> keys(n);
    cudaDeviceSynchronize();
    cudaError_t e = cudaMemcpy(keys.data(), g->shadow, n * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "grid_read_shadow");
    for (uint64_t i = 0; i < n; ++i) {
        if (keys[i] == ~0ull) {
            host[i] = 1.0f;
        } else {
            uint32_t b = uint32_t(keys[i] >> 32);
            std::memcpy(&host[i], &b, 4);
        }
    }
    return read_status(c);
}

int f184gi_grid_read_counts(f184gi_ctx* c, uint32_t grid, uint32_t* host) {
    if (!c || !host) return fail(F184GI_ERR_INVALID, "grid_read_counts: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_read_counts: unknown grid");
    if (!g->counts) return fail(F184GI_ERR_INVALID, "grid_read_counts: grid was created without F184GI_GRID_KEEP_COUNTS");
    cudaDeviceSynchronize();
    cudaError_t e = cudaMemcpy(host, g->counts, g->counts_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "grid_read_counts");
    return read_status(c);
}

int f184gi_grid_level_ptr(f184gi_ctx* c, uint32_t grid, uint32_t level, void** ptr, uint64_t* bytes) {
    if (!c || !ptr || !bytes) return fail(F184GI_ERR_INVALID, "grid_level_ptr: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_level_ptr: unknown grid");
    if (level >= g->desc.levels) return fail(F184GI_ERR_INVALID, "grid_level_ptr: level out of range");
    const ChainLayout& ch = g->chain;
    g->low_levels_current = false;  // the caller may write through the pointer: the next mip builds from L0
    *ptr = static_cast<char*>(ch.base) + ch.off[level] * ch.esz;
    *bytes = ch.vol[level] * ch.esz * ((ch.aniso && level > 0) ? 6 : 1);
    return F184GI_OK;
}

}  // extern "C"

namespace f184 {
// Device description of a grid for batched tracing (used by the request server).
int grid_internal(f184gi_ctx* c, uint32_t grid, ChainLayout* chain, const f184gi_grid_frame** d_frame) {
    if (!c || !chain || !d_frame) return fail(F184GI_ERR_INVALID, "grid_internal: null argument");
    GridObj* g = find_grid(c, grid);
    if (!g) return fail(F184GI_ERR_NOTFOUND, "grid_internal: unknown grid");
    *chain = g->chain;
    *d_frame = g->d_frame;
    return F184GI_OK;
}

int ctx_internal(f184gi_ctx* c, int* device, uint32_t** d_status) {
    if (!c || !device || !d_status) return fail(F184GI_ERR_INVALID, "ctx_internal: null argument");
    if (int rc0 = refused(c, "call")) return rc0;
    *device = c->device;
    *d_status = c->d_status;
    return F184GI_OK;
}

int ctx_status_capture(f184gi_ctx* c, uint32_t* host_pinned, cudaStream_t s) {
    if (!c || !host_pinned) return fail(F184GI_ERR_INVALID, "ctx_status_capture: null argument");
    cudaError_t e = cudaMemcpyAsync(host_pinned, c->d_status, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0, 4, s);
    return cuda_fail(e, "status capture");
}

int ctx_status_report(f184gi_ctx* c, uint32_t status) {
    if (!c) return fail(F184GI_ERR_INVALID, "ctx_status_report: null context");
    return decode_status(c, status);
}

void view_clip_matrix(const f184gi_view* v, double M[16]) {
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) {
            double acc = 0.0;
            for (int j = 0; j < 4; ++j) acc += double(v->proj[r * 4 + j]) * double(v->view[j * 4 + k]);
            M[r * 4 + k] = acc;
        }
}
}  // namespace f184
