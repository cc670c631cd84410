// gi_internal.h -- shared host-side declarations of the f184gi library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/f184gi.h"

namespace f184 {

constexpr int kMaxLevels = 11;
constexpr int kBrickEdge = 8;
constexpr int kBrickVox = 512;
constexpr uint32_t kFixedFrac = 31;  // per-contribution injection weights are 1.31 fixed point (64-bit sums)

// device status bits (set by kernels, read by f184gi_sync / inspection calls)
constexpr uint32_t kStatusOverflow = 1u;
constexpr uint32_t kStatusTimeout = 2u;
// View sides of 1..kMaxViewSide pixels; one trace call covers at most kMaxTracePixels pixels in all, so that its
// warp-tile numbering (32 pixels a tile) stays inside uint32.
constexpr uint32_t kMaxViewSide = 16384;
constexpr uint32_t kMaxRasterSide = 8192;  // rasterized images (shadow maps, G-buffers): 1/16-pixel snaps in range
constexpr uint64_t kMaxTracePixels = 1ull << 36;
constexpr uint32_t kStatusRange = 4u;      // geometry outside the fixed-point range was skipped
constexpr uint32_t kStatusNonFinite = 8u;  // triangles with a NaN or infinite coordinate were skipped
// a bounded wait on a bulk copy into shared memory expired: the CTA waited a second bounded window for its copy and
// returned, so the copy may still land in shared memory the SM has handed to another CTA.  The context that reads
// this bit refuses every later call (F184GI_ERR_TIMEOUT), so nothing it launches runs beside such a copy.
constexpr uint32_t kStatusCopyTimeout = 16u;

// process-wide count of kernels this library has launched (f184gi_kernel_launches)
void note_launches(uint32_t n);

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
bool invert4(const double* m, double* inv);

// The world -> L0 voxel map of a grid as FP32 pairs (h + l): p_voxel = (p - origin) * inv_vs.  Kept on the device
// right after the grid's frame (the frame kernel writes both), so the per-pixel trace reads floats only and runs
// no FP64.
struct FramePairs {
    float org_h[3], org_l[3];
    float ivs_h, ivs_l;
};
constexpr size_t kFrameAllocBytes = sizeof(f184gi_grid_frame) + sizeof(FramePairs);
// A grid's frame and its FP32 pairs as they lie on the device (computed on the host when the bounds are given).
struct FrameBlock {
    f184gi_grid_frame frame;
    FramePairs pairs;
};
static_assert(sizeof(FrameBlock) == kFrameAllocBytes, "the frame block is the frame followed by its pairs");
int compute_frame_block(const f184gi_bounds& b, uint32_t dim, const float light_dir[3], FrameBlock* out);
inline const FramePairs* frame_pairs(const f184gi_grid_frame* d_frame) {
    return reinterpret_cast<const FramePairs*>(d_frame + 1);
}

// Grid placement computed on the host in FP64 (same operation order as the device variant).
int compute_frame(const f184gi_bounds& b, uint32_t dim, const float light_dir[3], f184gi_grid_frame* out);

// Element layout of one grid's mip chain.  Level l has dim_l = dim >> l voxels per axis; levels with
// dim_l >= 8 are stored as 8^3 bricks in Morton order of the brick coordinates, voxels x-fastest inside a
// brick; smaller levels are linear.  Anisotropic chains store six direction volumes per level >= 1.
struct ChainLayout {
    void* base;
    uint32_t dim, levels, format, aniso;
    uint32_t esz;                    // bytes per voxel (16 F32, 8 F16)
    uint64_t off[kMaxLevels];        // element offset of level l (first direction volume)
    uint64_t vol[kMaxLevels];        // elements of one volume of level l
    uint32_t ldim[kMaxLevels];
};

// Host view of scratch memory used by one pass; grows on demand, kept by the context.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// ---- kernel launchers (defined in the .cu files) ----

struct RasterJob {
    const float* tri;       // 9 floats per triangle
    uint64_t ntris;
    double M[16];           // world -> clip (used when d_M is null)
    const double* d_M;      // world -> clip in device memory (e.g. a device-computed frame), or null
    uint32_t width, height;
    unsigned long long* keys;  // width*height, output
};
// bytes of scratch a raster job needs
size_t raster_scratch_bytes(uint64_t ntris, uint32_t width, uint32_t height);
int raster_launch(const RasterJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                  cudaStream_t s);

struct VoxelizeJob {
    const float* tri;
    const uint32_t* albedo;
    uint64_t ntris;
    const f184gi_grid_frame* d_frame;   // device copy of the frame
    f184gi_light light;
    ChainLayout chain;
    const unsigned long long* shadow_keys;
    uint32_t shadow_res;
    uint32_t* counts;                   // optional (dim^3, linear)
    const uint32_t* dirty_bricks;       // optional list (Morton brick indices of L0)
    uint32_t ndirty;
    float4* weights;                    // optional: write the mean-weight grid W instead of L0 radiance
    uint32_t mip_levels;                // with L0: also write levels 1 .. mip_levels (<= 3) of each brick's block
                                        // (isotropic FP32 chains; 0 = L0 only)
};
// L0 = luminance * (lit ? W : 0) over the whole grid (after a shadow-map change); W as written by voxelize
int relight_launch(const float4* weights, const f184gi_grid_frame* d_frame, const ChainLayout& chain,
                   const f184gi_light& light, const unsigned long long* shadow, uint32_t res, cudaStream_t s);
size_t voxelize_scratch_bytes(uint64_t ntris, uint32_t dim);
// Two phases: the triangle setup and (triangle, brick) lists, which do not read the shadow map, then the bricks
// (coverage, injection through the shadow map, L0 written).  The lists phase may run on another stream beside
// the shadow raster; the bricks phase must follow both (with resident weights it reads no shadow map and may
// follow the lists alone).
int voxelize_lists_launch(const VoxelizeJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                          cudaStream_t s);
int voxelize_bricks_launch(const VoxelizeJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                           cudaStream_t s);

// one bounded mbarrier wait that expires unless `complete` (the failure path of bounded device waits, on demand)
int bounded_wait_selftest_launch(uint32_t polls, uint32_t complete, uint32_t* status, cudaStream_t s);

// device-side frame from bounds (or from the triangles' AABB when bounds == nullptr)
int frame_launch(const float* tri, uint64_t ntris, const f184gi_bounds* bounds, uint32_t dim,
                 const float light_dir[3], f184gi_grid_frame* d_frame, void* scratch, cudaStream_t s);

// levels from+1 .. levels-1 from level `from` (0: the whole chain from L0)
int mip_launch(const ChainLayout& chain, uint32_t levels, uint32_t from, uint32_t* d_status, cudaStream_t s);

struct TraceView {
    float iview[16];                     // inverse view (FP32 of the FP64 inverse: normals)
    float iproj_h[16], iproj_l[16];      // FP64 inverse projection as FP32 pairs h + l (the float-float position)
    float iview_h[12], iview_l[12];      // rows 0..2 of the FP64 inverse view as FP32 pairs
    float eye[3];
    uint32_t width, height;
    const float* depth;
    const uint32_t* normal;
    const uint16_t* rough;
    void* out;
    uint32_t out_format;
    // the grid this view traces (batched launches mix grids)
    const void* grid_base;
    uint32_t grid_dim, grid_levels;
    const f184gi_grid_frame* frame;
    float tmax;
    uint64_t off[kMaxLevels], vol[kMaxLevels];
};
// The march schedule of the diffuse cones.  All diffuse cones start at start_offset with one aperture, so their
// k-th sample has the same distance t (a float pair t + tl), diameter and unclamped level log2(diameter) at every
// pixel; the host computes the first kDiffuseSched samples once per launch (trace_consts_schedule) and the
// kernel reads them instead of re-deriving them per cone and step.  Marches longer than the table continue with
// the same recurrence on the device.
constexpr uint32_t kDiffuseSched = 24;
struct SchedEntry {
    float t, tl, diam, lvl;  // lvl = max(log2(diam), 0), before the clamp to the grid's last level
};
struct TraceConsts {
    float tmax;
    float cos_tilt, sin_tilt;
    f184gi_cone_params p;
    SchedEntry sched[kDiffuseSched];
    unsigned long long* counts;  // the counting kernel's totals: cone steps, level samples (null otherwise)
};
void trace_consts_schedule(TraceConsts& tc);  // fills tc.sched from tc.p
// the FP64 inverse projection and inverse view split into FP32 pairs (the trace's float-float pixel set-up)
inline void trace_view_set_inverses(TraceView& t, const double IP[16], const double IV[16]) {
    for (int k = 0; k < 16; ++k) {
        t.iview[k] = float(IV[k]);
        t.iproj_h[k] = float(IP[k]);
        t.iproj_l[k] = float(IP[k] - double(t.iproj_h[k]));
    }
    for (int k = 0; k < 12; ++k) {
        t.iview_h[k] = float(IV[k]);
        t.iview_l[k] = float(IV[k] - double(t.iview_h[k]));
    }
}
// Cone-trace kernel variants: the tile shape (tw x th pixels, one thread each) and the CTAs kept resident per SM
// (the register budget).  Every variant computes each pixel with the same arithmetic, so results are identical;
// the batched launch picks the fastest by timing them on the work it serves.
struct TraceVariant {
    uint32_t tw, th, minb;  // CTA of tw x th pixels (warp tiles of tw x 32/tw), at least minb CTAs per SM
};
constexpr uint32_t kTraceVariantCount = 5;
constexpr TraceVariant kTraceVariants[kTraceVariantCount] = {
    {16, 8, 4}, {4, 24, 7}, {4, 32, 7}, {8, 16, 5}, {4, 24, 9}};
// The one-shot launch's variant (per 1080p view; the CTAs per SM set the register budget): 128-thread CTAs of
// 4x8-pixel warp tiles at 7 per SM (72 registers) for every chain: FP32 1.622 ms against 1.628 for 96-thread CTAs
// at 7 per SM (80 registers, 8 resident), FP16 1.848; the 512^3 anisotropic FP16 4K view 15.3 ms against 15.7 with
// 8x4 tiles at 5 per SM.  With every cone marched from one call site the pixel's state between cones goes to local
// memory at these budgets, reloaded once per cone.
constexpr uint32_t trace_default_variant(uint32_t fmt, bool aniso) {
    (void)fmt;
    (void)aniso;
    return 2u;
}
const void* trace_kernel_fn(uint32_t fmt, bool aniso, uint32_t variant);
const void* trace_kernel_count_fn(uint32_t fmt, bool aniso);  // instrumented, default variant's tile shape
uint32_t trace_view_tiles(uint32_t width, uint32_t height, uint32_t variant);
void trace_view_set_grid(TraceView& v, const ChainLayout& c, const f184gi_grid_frame* d_frame, float tmax);

// One-shot launch of one or more views of one grid (the view table goes through pinned staging).
struct TraceStaging;
void trace_staging_destroy(TraceStaging* st);
size_t trace_scratch_bytes(uint32_t nviews);
// count: launch the instrumented kernel (tc.counts set) with the default variant's shape
int trace_launch(const ChainLayout& chain, const TraceConsts& tc, const f184gi_grid_frame* d_frame,
                 const TraceView* views, uint32_t nviews, void* scratch, size_t scratch_bytes, uint32_t variant,
                 TraceStaging** staging, cudaStream_t s, bool count = false);

// Batched trace replayed from CUDA graphs: [view table H2D] -> [work counter = 0] -> [kernel over all views].
struct TraceGraph;
uint32_t trace_persistent_blocks(uint32_t fmt, bool aniso, uint32_t variant, uint32_t per_sm);  // per_sm 0 = max
int trace_graph_create(TraceGraph** out, uint32_t fmt, bool aniso, uint32_t max_views, uint32_t per_sm,
                       const TraceConsts& tc);
int trace_graph_launch(TraceGraph* g, const TraceView* views, uint32_t nviews, uint32_t variant, cudaStream_t s);
// time every variant on this batch (outputs are written each time, identically); the fastest goes to *best
int trace_graph_tune(TraceGraph* g, const TraceView* views, uint32_t nviews, cudaStream_t s, uint32_t* best,
                     float* ms);
void trace_graph_destroy(TraceGraph* g);

// Reference-faithful volume and march (march.cu)
size_t refvox_scratch_bytes(uint64_t ntris, uint32_t dim);
int refvox_launch(const float* tri, const uint32_t* albedo, uint64_t ntris, const f184gi_grid_frame* d_frame,
                  uint32_t dim, uint32_t* vol, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                  cudaStream_t s);
struct MarchJobDev {
    f184gi_march_params p;
    const uint32_t* vol;
    const unsigned long long* shadow;
    const f184gi_grid_frame* frame_ptr;
    uint32_t dim, res;
    float lum[3], light_dir[3];
    float pow5[32], pow6[64];  // (k / 31)^2.2 and (k / 63)^2.2, the 565 albedo decode (indirect.frag:157)
};
struct MarchViewDev {
    float iview[16], iproj[16];
    double iproj_zw[8];
    uint32_t width, height;
    const float* depth;
    const uint32_t* normal;
    void* out;
};
int march_launch(const MarchJobDev& job, const MarchViewDev& view, cudaStream_t s);

// cross-bilateral blur of an RGBA FP32 image (two passes through tmp)
int blur_launch(const float* in, const float* depth, uint32_t W, uint32_t H, float* tmp, float* out, cudaStream_t s);

// grid of a context as the kernels see it (chain layout and device frame)
int grid_internal(f184gi_ctx* c, uint32_t grid, ChainLayout* chain, const f184gi_grid_frame** d_frame);
// the context's device ordinal and device status word
int ctx_internal(f184gi_ctx* c, int* device, uint32_t** d_status);
// Stream-ordered status: copy the context's device status word to pinned host memory and clear it, on stream s
// (ordered after the work issued before it); then decode a captured word as f184gi_sync would report it.
int ctx_status_capture(f184gi_ctx* c, uint32_t* host_pinned, cudaStream_t s);
int ctx_status_report(f184gi_ctx* c, uint32_t status);
// clip = proj * view of a view in FP64, summed in index order without FMA contraction
void view_clip_matrix(const f184gi_view* v, double M[16]);

int gbuffer_resolve_launch(const unsigned long long* keys, uint32_t width, uint32_t height, const float* tri,
                           const float* rough, const float view[16], const float eye[3], float* depth,
                           uint32_t* normal, uint16_t* rough_out, uint32_t* tri_out, cudaStream_t s);

int read_level_launch(const ChainLayout& chain, uint32_t level, uint32_t dir, float* d_out, cudaStream_t s);

// translate triangle ranges (FP32 adds, the same rounding as a host-side mirror)
int moves_launch(float* tri, const f184gi_move* moves, uint32_t nmoves, cudaStream_t s);

// dst = model (row-major 3x4) * src, per vertex; products and sums rounded in order (no FMA)
int transform_launch(const float* src, uint64_t ntris, const float model[12], float* dst, cudaStream_t s);

}  // namespace f184
