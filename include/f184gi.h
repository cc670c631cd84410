/*
 * f184gi.h -- C ABI of the GB300 voxel global-illumination path.
 *
 * The path has three passes, driven in the same order as the reference renderer's frame:
 *   f184gi_voxelize  -- shadow map + conservative voxelization with direct-light injection
 *                       (replaces CZOnlyRenderer::RenderList, Foreground/Renderer/ZOnlyRenderer.h:21-22,
 *                        and CVoxelizeRenderer::RenderList, Foreground/Renderer/VoxelizeRenderer.h:21-22,
 *                        as called from CMegaPipeline::Render, Foreground/Renderer/MegaPipeline.cpp:188-223)
 *   f184gi_mip       -- 3D mip chain of the radiance/opacity grid (the reference volume has one level,
 *                       Foreground/Renderer/MegaPipeline.cpp:474-482; this pass has no reference counterpart)
 *   f184gi_trace     -- per-pixel diffuse + specular cone trace over a G-buffer
 *                       (replaces the lighting_indirect fullscreen pass, Foreground/Renderer/MegaPipeline.cpp:241-268,
 *                        shader Shader/Lighting/indirect.frag:104-243)
 *
 * Conventions
 *  - Every entry point returns an int status: 0 = ok, negative = error; f184gi_last_error() returns a
 *    thread-local message for the last failure on the calling thread.
 *  - Buffers passed as `const float*` etc. to the pass calls are DEVICE pointers unless the name says host.
 *    Work is stream-ordered on the caller's cudaStream_t, passed as `void*` (NULL = legacy default stream).
 *  - Matrices are row-major 4x4 floats acting on column vectors (v' = M v), the memory layout of
 *    tc::Matrix4 (Math/Matrix4.h).  The reference transposes them before upload to GLSL
 *    (Foreground/SceneGraph/SceneView.cpp:28-30); this ABI takes them untransposed.
 *  - One context owns its device buffers; it is not thread-safe (like CMegaPipeline, MegaPipeline.cpp:374-375):
 *    callers serialise calls on one context.  Separate contexts may be used from separate threads.
 */
#ifndef F184GI_H
#define F184GI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define F184GI_ABI_VERSION 1

/* status codes */
#define F184GI_OK 0
#define F184GI_ERR_INVALID (-1)  /* bad argument (null pointer, size out of range, unknown handle) */
#define F184GI_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define F184GI_ERR_OOM (-3)      /* device allocation failed */
#define F184GI_ERR_BUDGET (-4)   /* request does not fit the context's HBM budget */
#define F184GI_ERR_OVERFLOW (-5) /* a bounded device structure overflowed (result invalid) */
#define F184GI_ERR_TIMEOUT (-6)  /* a bounded wait expired */
#define F184GI_ERR_NOTFOUND (-7) /* unknown grid / request id */
#define F184GI_ERR_CANCELLED (-8)
#define F184GI_ERR_WORKER (-9)   /* a server's scheduler thread stopped: its queued requests fail, new ones are refused */

/* ---- boundary value types (layout-compatible with the reference Math library) ---- */

/* tc::Vector3 (Math/Vector3.h), 12 bytes */
typedef struct f184gi_vec3 {
    float x, y, z;
} f184gi_vec3;

/* tc::BoundingBox (Math/BoundingBox.h:321-325): Min, pad, Max, pad -- 32 bytes */
typedef struct f184gi_bounds {
    f184gi_vec3 min;
    float pad0;
    f184gi_vec3 max;
    float pad1;
} f184gi_bounds;

/* The sun as the reference binds it (PerLightConstants, MegaPipeline.cpp:95-99, 264-265):
 * luminance = Color * Intensity (Foreground/SceneGraph/Light.h:18),
 * direction = the light node's world -Z (MegaPipeline.cpp:110), i.e. the direction light travels.
 * Lambert uses -direction (indirect.frag:167). */
typedef struct f184gi_light {
    float luminance[3];
    float direction[3];
} f184gi_light;

/* storage formats of the radiance/opacity grid (RGB = radiance premultiplied by opacity, A = opacity) */
#define F184GI_FMT_F32 0u /* float4 per voxel, 16 B */
#define F184GI_FMT_F16 1u /* 8 B per voxel: R, G, B as IEEE binary16 and opacity as 16-bit unorm (n / 65535); as
                          * a trace output format: half4 */
#define F184GI_FMT_RG16 2u /* the reference's voxel volume (one level): uint32 per voxel = RGB565 albedo in the low
                            * 16 bits, the 5-6-5 packed normal in the high 16 (main.lua:269-272); for f184gi_march */

/* grid flags */
#define F184GI_GRID_KEEP_COUNTS 1u /* also keep the per-voxel contribution count (u32, L0) for inspection */
/* Keep the unshadowed mean injection weight of every voxel (FP32 RGBA, 16 B/voxel) resident.  f184gi_voxelize
 * then re-voxelizes only the dirty bricks' geometry and relights the whole grid from the new shadow map, so a
 * moved object's shadow changes propagate without re-voxelizing the bricks it shadows.  L0 is byte-identical to
 * a full voxelization. */
#define F184GI_GRID_RESIDENT_WEIGHTS 2u

typedef struct f184gi_grid_desc {
    uint32_t dim;         /* voxels per axis at L0: power of two, 16..512 */
    uint32_t levels;      /* mip levels including L0: 1..log2(dim) */
    uint32_t format;      /* F184GI_FMT_* */
    uint32_t anisotropic; /* 0 = isotropic mips, 1 = 6-direction anisotropic mips (levels >= 1) */
    uint32_t shadow_res;  /* shadow map texels per side: 64..8192 */
    uint32_t flags;       /* F184GI_GRID_* */
} f184gi_grid_desc;

/* Placement of the grid in the world, derived from the scene bounds in FP64 (read back with f184gi_grid_get_frame).
 * voxel v = floor((p - origin) / voxel_size). */
typedef struct f184gi_grid_frame {
    double origin[3];
    double voxel_size;
    double inv_voxel_fixed; /* 256 / voxel_size: world -> 24.8 voxel fixed point */
    double light_clip[16];  /* world -> shadow clip space (row-major), z in [0,1] */
    double shadow_bias;     /* clip-z bias of the shadow compare (two voxels along the light) */
    double light_dir[3];    /* normalised direction of travel */
    /* shadow clip coordinates of voxel centres as FP32 affine functions of the voxel index:
     * row r in (x, y, z): light_vox[4r] + i light_vox[4r+1] + j light_vox[4r+2] + k light_vox[4r+3] */
    float light_vox[12];
    float shadow_bias_f;
    float pad_f[3];
} f184gi_grid_frame;

/* One view over one G-buffer (the trace's inputs).  The G-buffer layout:
 *   depth     FP32 per pixel, NDC depth of `proj` (the value the reference's depth attachment holds,
 *             decoded with InvProj as indirect.frag:50-55 does); >= 1.0 marks background.
 *   normal    2 x FP16 per pixel (packed in a u32, low half = x): octahedral encoding of the view-space
 *             unit normal (the reference stores view-space normals, Pipelang/Internal/main.lua:56).
 *   roughness FP16 per pixel (the reference's Target2.g, main.lua:238).
 * Row y = 0 is the top of the image (uv.y = (y + 0.5) / height, as the reference's fullscreen pass). */
typedef struct f184gi_view {
    float view[16]; /* world -> view, row-major */
    float proj[16]; /* view -> clip, row-major (CCamera::CalcPerspective convention) */
    uint32_t width, height; /* 1..16384 each (1..8192 for f184gi_gbuffer); a trace call or served batch covers
                             * at most 2^36 pixels */
    const float* depth;
    const uint32_t* normal;
    const uint16_t* roughness;
    void* out;           /* 2 * width * height RGBA: [diffuse.rgb, occlusion] then [specular.rgb, alpha] */
    uint32_t out_format; /* F184GI_FMT_F32 (float4) or F184GI_FMT_F16 (half4) */
    uint32_t pad;
} f184gi_view;

/* Cone-trace parameters; f184gi_cone_params_default fills the defaults noted below. */
typedef struct f184gi_cone_params {
    uint32_t diffuse_cones;  /* 5 (1 along the normal + 4 tilted) or 1 */
    float diffuse_tan_half;  /* tan(30 deg): 60-degree aperture */
    float diffuse_tilt_deg;  /* 60: tilt of the side cones from the normal */
    float step_factor;       /* 0.5: step = step_factor * cone diameter */
    float max_distance;      /* in L0 voxels; <= 0 means the grid diagonal */
    float alpha_stop;        /* 1.0: stop a cone once its opacity reaches this (1.0 = only when opaque; a lower
                              * threshold makes the result jump where rounding moves the crossing by a step) */
    float start_offset;      /* 1.0: origin offset along the normal, in L0 voxels */
    float min_spec_tan_half; /* 0.05: specular cone tan(half aperture) = max(roughness, this) */
    uint32_t specular;       /* 1 = trace the specular cone */
    uint32_t pad;
} f184gi_cone_params;

typedef struct f184gi_config {
    int device;              /* CUDA device ordinal */
    uint32_t flags;
    uint64_t hbm_budget;     /* bytes the context may hold on the device; 0 = no limit */
} f184gi_config;

typedef struct f184gi_ctx f184gi_ctx;

/* ---- context and grids ---- */
const char* f184gi_last_error(void);
int f184gi_abi_version(void);
/* number of kernels this library has launched in this process (diagnostics) */
uint64_t f184gi_kernel_launches(void);
/* Diagnostic, with no counterpart in the reference: one device wait on a shared-memory mbarrier, bounded to
 * `polls` polls (1..2^24), whose phase completes only when `complete` is 1.  An expired wait is recorded in the
 * context's status exactly as the library's own bounded waits record theirs, so the next f184gi_sync returns
 * F184GI_ERR_TIMEOUT and the context stays usable: the failure path, exercised without a GPU fault.  With
 * `complete` = 2 the expired wait is recorded as the mip pass records an expired wait on its bulk copy (no copy is
 * involved here): the next f184gi_sync returns F184GI_ERR_TIMEOUT and the context refuses every later call. */
int f184gi_selftest_bounded_wait(f184gi_ctx* ctx, uint32_t polls, uint32_t complete, void* stream);
int f184gi_create(const f184gi_config* cfg, f184gi_ctx** out);
int f184gi_destroy(f184gi_ctx* ctx);
/* bytes currently held on the device by the context */
int f184gi_memory_used(f184gi_ctx* ctx, uint64_t* bytes);

/* Allocate a radiance/opacity grid with its mip chain and shadow map.  Grids stay resident until destroyed. */
int f184gi_grid_create(f184gi_ctx* ctx, const f184gi_grid_desc* desc, uint32_t* grid);
int f184gi_grid_destroy(f184gi_ctx* ctx, uint32_t grid);
/* bytes a grid with this descriptor occupies (grid + mips + shadow map + scratch reserve) */
int f184gi_grid_bytes(const f184gi_grid_desc* desc, uint64_t* bytes);

/* ---- the three passes ---- */

/* Voxelize `ntris` triangles (tri_xyz: 9 floats per triangle, device) with per-triangle RGBA8 albedo
 * (device, R in the low byte) into `grid`, injecting the directional light through a shadow map that this
 * call rasterizes.  bounds (host pointer) fixes the grid placement; NULL = the triangles' own AABB,
 * reduced on the device.  dirty_bricks (device, brick indices in Morton order) limits the rewrite to those
 * 8^3 bricks of L0 (ndirty = 0: whole grid); the shadow map is always rebuilt.  Isotropic FP32 grids without
 * resident weights also get each rewritten brick's block of levels 1..3 (the mip values of L0), so the next
 * f184gi_mip continues from level 3 with the same bytes as a build from L0. */
int f184gi_voxelize(f184gi_ctx* ctx, uint32_t grid, const float* tri_xyz, const uint32_t* albedo,
                    uint64_t ntris, const f184gi_bounds* bounds, const f184gi_light* light,
                    const uint32_t* dirty_bricks, uint32_t ndirty, void* stream);

/* Build mip levels 1..levels-1 from L0 (levels = 0: all levels of the grid). */
int f184gi_mip(f184gi_ctx* ctx, uint32_t grid, uint32_t levels, uint32_t anisotropic, void* stream);

/* Cone-trace every pixel of every view against `grid`; params NULL = defaults. */
int f184gi_trace(f184gi_ctx* ctx, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                 const f184gi_cone_params* params, void* stream);

void f184gi_cone_params_default(f184gi_cone_params* p);

/* Diagnostic, with no counterpart in the reference: the same trace as f184gi_trace (same outputs) through an
 * instrumented kernel that also counts, over all pixels of all views, the cone steps (counts[0]) and the level
 * samples (counts[1]; a step samples one mip level or two, 8 voxel taps each).  counts is a host array; the
 * call waits for the stream.  Slower than f184gi_trace: for stating the sampled-bytes figure of a trace. */
int f184gi_trace_count(f184gi_ctx* ctx, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                       const f184gi_cone_params* params, uint64_t counts[2], void* stream);

/* ---- supporting passes ---- */

/* A rigid move of one object: triangles [first, first + count) translated by offset (FP32 adds per vertex). */
typedef struct f184gi_move {
    uint32_t first, count;
    float offset[3];
} f184gi_move;

/* Apply moves to a device triangle buffer of ntris triangles (moves: host array). */
int f184gi_apply_moves(f184gi_ctx* ctx, float* tri_xyz, const f184gi_move* moves, uint32_t nmoves, uint64_t ntris,
                       void* stream);

/* world_xyz = model * obj_xyz for ntris triangles (9 floats each, device buffers), model = a row-major 3x4
 * matrix in the layout of tc::Matrix3x4 (Math/Matrix3x4.h).  This is the per-primitive ModelMat transform the
 * reference applies in its voxelization geometry stage (Pipelang/Internal/main.lua:94-98, 130-131). */
int f184gi_transform(f184gi_ctx* ctx, const float* obj_xyz, uint64_t ntris, const float model[12], float* world_xyz,
                     void* stream);

/* Rasterize a G-buffer for one camera (the reference's GBufferRenderer pass,
 * Foreground/Renderer/GBufferRenderer.cpp:79-116 with main.lua:32-58,227-240): flat face normals facing the
 * camera, per-triangle roughness (device FP32), depth of view->proj.  Writes view->depth/normal/roughness
 * (device buffers owned by the caller).  Fragment ties resolve to the lowest triangle index. */
int f184gi_gbuffer(f184gi_ctx* ctx, const float* tri_xyz, const float* roughness, uint64_t ntris,
                   const f184gi_view* view, uint32_t* tri_id_out, void* stream);

/* f184gi_gbuffer without any device allocation; no counterpart in the reference.  For callers that cannot
 * allocate device memory while they draw: a render loop that must not stall on the device-wide synchronisation
 * of cudaMalloc/cudaFree, or a process whose device memory is all handed out (to a caching allocator, or to a
 * context at its HBM budget).  Same arguments and results as f184gi_gbuffer; the scratch is one fixed 48 MiB
 * device array in the library, shared by every call on a device.  Limits: ntris <= 262144 and
 * width*height <= 2097152 (1920x1080 fits); larger calls return F184GI_ERR_INVALID and name the limit.  The
 * first call on a device looks up the array's address (and can load its module): make it before any stream
 * capture.  Calls that overlap on the GPU race on the array; calls in order on one stream do not.  Errors that
 * kernels flag are reported by f184gi_sync(ctx, stream) as for f184gi_gbuffer.  The call runs on the context's
 * device and restores the caller's current device.  The array's 48 MiB per device are counted neither in
 * f184gi_memory_used nor in a server's HBM budget; they are reserved when the library's module holding it loads
 * on a device (at the first call under CUDA's lazy module loading, at start-up under CUDA_MODULE_LOADING=EAGER). */
int f184gi_gbuffer_static(f184gi_ctx* ctx, const float* tri_xyz, const float* roughness, uint64_t ntris,
                          const f184gi_view* view, uint32_t* tri_id_out, void* stream);

/* Parameters of the reference-faithful march (indirect.frag:104-222); f184gi_march_params_default fills the
 * reference's constants noted below. */
typedef struct f184gi_march_params {
    uint32_t rays;          /* 4 rays per pixel (indirect.frag:202-218) */
    uint32_t second_bounce; /* 1: a ray that hits marches once more from the hit (indirect.frag:197) */
    uint32_t max_steps;     /* 60 steps per ray (indirect.frag:138) */
    uint32_t frame;         /* seed of the per-pixel random numbers (the reference's frameCount) */
    float step_size;        /* 0.2 world units (indirect.frag:116) */
    float normal_offset;    /* 0.06: shadow lookup pushed along the voxel normal (indirect.frag:161) */
    float shadow_bias;      /* 0.005 in shadow clip depth (indirect.frag:165) */
    float sky[3];           /* 0.7, 0.8, 1.0 (indirect.frag:180) */
    float sky_scale;        /* 0.4 */
    float pad;
} f184gi_march_params;
void f184gi_march_params_default(f184gi_march_params* p);

/* The reference-faithful indirect pass over an F184GI_FMT_RG16 grid that f184gi_voxelize filled (its shadow map
 * and light included): per pixel 4 rays with a second bounce, fixed steps, first-hit sun light behind the
 * shadow map, sky for rays that take every step.  Writes width*height RGBA FP32 to view->out:
 * [indirect.rgb, view-space distance] (the reference's outColor before its temporal blend, which is not
 * restated).  The reference's frame-dependent sin-hash noise is replaced by an integer hash of (pixel, frame,
 * ray).  roughness and out_format of the views are not used. */
int f184gi_march(f184gi_ctx* ctx, uint32_t grid, const f184gi_view* views, uint32_t nviews,
                 const f184gi_march_params* params, void* stream);

/* The reference's depth-aware blur of the indirect image (blurX then blurY over
 * Shader/Lighting/bilateralBlur.inc:19-73, MegaPipeline.cpp:270-284): rgba_in and rgba_out are width*height
 * RGBA FP32 device images (rgb blurred, out alpha 0), depth the G-buffer's FP32 depth.  rgba_out may not alias
 * rgba_in; the intermediate pass uses the context's scratch. */
int f184gi_blur(f184gi_ctx* ctx, const float* rgba_in, const float* depth, uint32_t width, uint32_t height,
                float* rgba_out, void* stream);

/* Wait for the stream, then report (and clear) errors that kernels flagged on the device since the last
 * check: F184GI_ERR_OVERFLOW (a bounded structure overflowed), F184GI_ERR_TIMEOUT (a bounded wait expired). */
int f184gi_sync(f184gi_ctx* ctx, void* stream);

/* ---- served form: continuous batching over device-resident grids ----
 *
 * A server owns resident scenes (triangles on the device + a grid with resident weights) and runs a request loop:
 * requests (rigid object moves + a set of views) queue on the host; whenever one of `slots` in-flight batches
 * is free, the scheduler admits pending requests (one per scene per batch, HBM budget for their staging
 * buffers, at most max_batch_views views), re-voxelizes the moved objects' bricks, relights and rebuilds the
 * mips of each touched scene, and traces every view of the batch in one launch replayed from a CUDA
 * graph.  Requests that arrive while batches run join the next batch; batches on different slots overlap.  A
 * scene's next request may be admitted while a batch holding the scene is in flight: its batch's update of the
 * scene waits (on the device) for that batch to finish.  Results are the same as running each request alone
 * (per scene, requests apply in submission order).  The f184gi_server_* calls on one server may come from several
 * host threads at once. */
typedef struct f184gi_server f184gi_server;

typedef struct f184gi_server_config {
    int device;
    uint32_t slots;           /* batches in flight (1..4, 0 = 2) */
    uint32_t max_batch_views; /* views per batched launch (0 = 64) */
    uint32_t blocks_per_sm;   /* 0: one trace warp per 32-pixel tile; k: a persistent wave of k CTAs per SM */
    uint64_t hbm_budget;      /* bytes for resident scenes + request staging (0 = no limit) */
    f184gi_cone_params cone;  /* cone parameters for every request (diffuse_cones == 0: defaults) */
    uint32_t trace_variant;   /* 0 = tune the cone-trace kernel variant on the first batch; k = use variant k-1 */
    uint32_t pad;
} f184gi_server_config;

#define F184GI_REQ_HOST_BUFFERS 1u /* view G-buffers / outputs are host pointers: staged through the budget */
/* Host-side fault injection (test hooks; no GPU fault is involved):
 *   INJECT_FAIL: this request's scene update fails with F184GI_ERR_CUDA before any of its device work is issued, as
 *     if a CUDA call had failed; the other requests of its batch run and the server keeps serving;
 *   INJECT_WORKER_EXIT: the scheduler thread exits after admitting the batch that holds this request, before
 *     issuing it (a worker lost between stages): that batch and every queued request fail with F184GI_ERR_WORKER,
 *     batches already on the device complete, and later submissions are refused with F184GI_ERR_WORKER. */
#define F184GI_REQ_INJECT_FAIL 0x100u
#define F184GI_REQ_INJECT_WORKER_EXIT 0x200u

typedef struct f184gi_request {
    uint32_t scene_id;
    uint32_t flags;
    const f184gi_move* moves; /* applied before the views are traced */
    uint32_t nmoves;
    uint32_t nviews;
    const f184gi_view* views;
} f184gi_request;

typedef struct f184gi_request_result {
    int status;         /* 0, F184GI_ERR_CANCELLED, or the failing call's status */
    uint32_t batch;     /* batch sequence number it ran in */
    double queued_ms;   /* submit -> admission */
    double latency_ms;  /* submit -> results complete on the device */
    uint64_t pixels;
} f184gi_request_result;

typedef struct f184gi_server_stats {
    uint64_t requests_done, requests_cancelled, batches, pixels;
    double p50_ms, p99_ms, mean_ms;  /* request latency over completed requests */
    double mean_batch_views;
    uint64_t hbm_used, hbm_budget;
    uint32_t pending, inflight;
    /* the cone-trace kernel variant the server tuned on its first batch: tile of trace_tile[0] x trace_tile[1]
     * pixels, trace_ctas_per_sm CTAs resident per SM; tune_ms = time of the first batch under each variant
     * (trace_variants entries used, 0 before tuning) */
    uint32_t trace_variant, trace_variants, trace_tile[2], trace_ctas_per_sm, pad;
    float tune_ms[8];
} f184gi_server_stats;

int f184gi_server_create(const f184gi_server_config* cfg, f184gi_server** out);
int f184gi_server_destroy(f184gi_server* s);
/* Register a scene: host triangles/albedo are copied to the device, voxelized and mip-mapped (synchronously). */
int f184gi_server_add_scene(f184gi_server* s, uint32_t scene_id, const f184gi_grid_desc* desc, const float* tri_xyz,
                            const uint32_t* albedo, uint64_t ntris, const f184gi_bounds* bounds,
                            const f184gi_light* light);
/* Queue a request (moves and views are copied); returns a ticket.  F184GI_ERR_BUDGET if its staging can never fit. */
int f184gi_server_submit(f184gi_server* s, const f184gi_request* req, uint64_t* ticket);
/* Queue n requests at once (all or none): the scheduler sees them together, so they can share one batch.
 * tickets[k] receives request k's ticket. */
int f184gi_server_submit_batch(f184gi_server* s, const f184gi_request* reqs, uint32_t n, uint64_t* tickets);
/* Wait until the ticket completes (timeout_ms 0 = no limit): F184GI_ERR_TIMEOUT when the wait expires. */
int f184gi_server_wait(f184gi_server* s, uint64_t ticket, uint32_t timeout_ms, f184gi_request_result* out);
/* Cancel a request that has not been admitted yet (F184GI_ERR_INVALID once it is running or done). */
int f184gi_server_cancel(f184gi_server* s, uint64_t ticket);
int f184gi_server_get_stats(f184gi_server* s, f184gi_server_stats* out);
/* Per-request metrics: one JSON line per finished request (ticket, scene, status, batch, views, pixels, queued and
 * latency ms) appended to `path` (NULL closes the log).  No counterpart in the reference (stdout only,
 * MegaPipeline.cpp:76). */
int f184gi_server_set_log(f184gi_server* s, const char* path);

/* ---- inspection (host copies; synchronise the stream) ---- */
int f184gi_grid_get_frame(f184gi_ctx* ctx, uint32_t grid, f184gi_grid_frame* out);
/* level as linear FP32 RGBA, x fastest: dim_l^3 * 4 floats (anisotropic: direction `dir` 0..5 for level >= 1) */
int f184gi_grid_read_level(f184gi_ctx* ctx, uint32_t grid, uint32_t level, uint32_t dir, float* host_rgba);
/* shadow map as FP32 depth (1.0 = empty), shadow_res^2 floats, row 0 first */
int f184gi_grid_read_shadow(f184gi_ctx* ctx, uint32_t grid, float* host_depth);
/* per-voxel contribution counts at L0 (needs F184GI_GRID_KEEP_COUNTS), linear x fastest */
int f184gi_grid_read_counts(f184gi_ctx* ctx, uint32_t grid, uint32_t* host_counts);
/* device pointer and byte size of one level (for callers that sample the chain themselves).  Layout: level 0 in
 * 8^3 bricks (voxels x fastest) in Morton order of brick coordinates; levels >= 1 linear, x fastest, inside a
 * one-voxel ring of zeros ((d + 2)^3 elements; voxel (x, y, z) at ((z + 1) (d + 2) + y + 1) (d + 2) + x + 1);
 * anisotropic levels hold six such volumes (+x, -x, +y, -y, +z, -z) back to back.  The caller may write through
 * the pointer: the grid's next f184gi_mip then builds every level from L0. */
int f184gi_grid_level_ptr(f184gi_ctx* ctx, uint32_t grid, uint32_t level, void** dev_ptr, uint64_t* bytes);

/* Host computation of the grid frame that f184gi_voxelize derives from `bounds` (bit-identical to it). */
int f184gi_frame_from_bounds(const f184gi_bounds* bounds, uint32_t dim, const float light_dir[3],
                             f184gi_grid_frame* out);

/* ---- host helpers mirroring Foreground/SceneGraph/Camera.cpp ---- */
/* CCamera::CalcPerspective (Camera.cpp:85-102): fovy in degrees */
void f184gi_camera_perspective(float fovy_deg, float aspect, float near_clip, float far_clip, float out[16]);
/* CCamera::CalcOrtho (Camera.cpp:104-111) */
void f184gi_camera_ortho(float mag_x, float mag_y, float near_clip, float far_clip, float out[16]);
/* view matrix of a camera at `eye` looking at `target` with +Y up: the inverse of the camera node's world
 * transform (SceneView.cpp:28), camera looking down its local -Z */
void f184gi_camera_look_at(const float eye[3], const float target[3], float out[16]);
/* general 4x4 inverse (FP64 internally); returns 0, or F184GI_ERR_INVALID when singular */
int f184gi_mat4_inverse(const float m[16], float out[16]);

/* ---- seeded synthetic scenes (host memory owned by the library) ---- */
typedef struct f184gi_scene {
    uint64_t ntris;
    uint32_t nobjects;
    uint32_t pad;
    float* tri_xyz;           /* 9 floats per triangle */
    uint32_t* albedo;         /* RGBA8 per triangle */
    float* roughness;         /* per triangle, uniform [0.1, 0.9] */
    uint32_t* object_first;   /* first triangle of each object (room = object 0) */
    uint32_t* object_count;   /* triangles per object */
    f184gi_bounds bounds;
    f184gi_light light;
    float eye[3], target[3];  /* seeded camera inside the room */
} f184gi_scene;

/* Load a glTF 2.0 scene (.gltf with buffers beside it or in data URIs, or .glb) as world-space triangles: the
 * default scene's node tree (matrix or T*R*S composed with the parent), triangle primitives (lists, strips,
 * fans; u8/u16/u32 or no indices), one object per (node, primitive), per-triangle albedo = baseColorFactor
 * (RGBA8, default white) and roughness = roughnessFactor (default 1).  Replaces the reference's importer
 * (Foreground/SceneGraph/glTFSceneImporter.cpp:200-440), which returns silently on a bad file; here
 * F184GI_ERR_NOTFOUND / F184GI_ERR_INVALID with the reason.  Light = the reference's sun
 * (f184gi_reference_sun_direction, App/MainBehaviour.cpp:40-44), camera outside the bounds looking at the centre.
 * Free with f184gi_scene_free. */
int f184gi_gltf_load(const char* path, f184gi_scene** out);
/* Direction of travel of the reference's sun: -Z of a node rotated by the Euler angles (-75, -30, 50) degrees. */
void f184gi_reference_sun_direction(float dir[3]);

/* Room (6 quads bounding [-10,10]^3) + nobjects boxes/UV-spheres (half each) with ~target_tris triangles
 * in total, seeded by `seed` (splitmix64 -> xoshiro256**). */
int f184gi_scene_generate(uint64_t seed, uint64_t target_tris, uint32_t nobjects, f184gi_scene** out);
void f184gi_scene_free(f184gi_scene* scene);
/* Rigidly move `fraction` of the objects (seeded) by up to `max_offset` world units; the moved objects'
 * indices go to moved_out (capacity nobjects), their count to nmoved. */
int f184gi_scene_move_objects(f184gi_scene* scene, uint64_t seed, float fraction, float max_offset,
                              uint32_t* moved_out, uint32_t* nmoved);
/* view i of a seeded camera path inside the room */
int f184gi_scene_camera(const f184gi_scene* scene, uint64_t seed, uint32_t i, float eye[3], float target[3]);

#ifdef __cplusplus
}
#endif

#endif /* F184GI_H */
