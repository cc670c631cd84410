/*
 * oracle.h -- CPU restatement of the voxel GI path.  TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker for the CUDA path: only the test suite, the smoke check and the CPU-baseline
 * leg of the benchmark load it.  The product library never links or calls it.
 *
 * Every function exists in two precisions: *_f64 is the correctness oracle, *_f32 the same code
 * instantiated in FP32, which the benchmark times as the CPU baseline.  Discrete decisions (raster coverage,
 * conservative voxel overlap, shadow visibility) are made in exact integer / IEEE-FP64 arithmetic with a
 * fixed operation order in both instantiations, so they do not depend on T.
 *
 * Parity is unpinned by the reference for the mip chain and the cone trace (the reference has neither:
 * Foreground/Renderer/MegaPipeline.cpp:481 allocates one level and Shader/Lighting/indirect.frag:104-184 marches
 * single rays); those follow the published voxel-cone-tracing method (Crassin et al. 2011).
 */
#ifndef F184GI_ORACLE_H
#define F184GI_ORACLE_H

#include <stdint.h>

#include "../include/f184gi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Grid placement + light frame (FP64), the same definition the product uses. */
int orc_grid_frame(const f184gi_bounds* bounds, uint32_t dim, const float light_dir[3], f184gi_grid_frame* out);

/* Exact triangle raster: u64 key = (float bits of depth) << 32 | triangle index, min per pixel
 * (~0 = empty).  clip = M * (x,y,z,1) in FP64; clipped to 0<=z<=w, |x|,|y| <= 16 w; vertices snapped to
 * 1/16 pixel; inclusive int64 edge functions at pixel centres; depth from the FP32-rounded plane
 * z0 + a dX + b dY evaluated in FP32 in that order. */
int orc_raster(const double M[16], uint32_t width, uint32_t height, const float* tri_xyz, uint64_t ntris,
               uint64_t* keys, int nthreads);

/* G-buffer resolve (f64): depth / octahedral view normal (FP16x2) / roughness (FP16) / triangle id */
int orc_gbuffer_resolve(const uint64_t* keys, uint32_t width, uint32_t height, const float* tri_xyz,
                        const float* roughness, const float view[16], float* depth, uint32_t* normal,
                        uint16_t* rough_out, uint32_t* tri_out);

/* Conservative voxelization + injection.  shadow_depth: res^2 FP32 (1.0 = empty).
 * rgba: dim^3 * 4 values, linear x fastest.  counts (optional): dim^3 contribution counts. */
int orc_voxelize_f64(const f184gi_grid_frame* frame, uint32_t dim, uint32_t shadow_res, const float* tri_xyz,
                     const uint32_t* albedo, uint64_t ntris, const f184gi_light* light,
                     const float* shadow_depth, double* rgba, uint32_t* counts, int nthreads);
int orc_voxelize_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t shadow_res, const float* tri_xyz,
                     const uint32_t* albedo, uint64_t ntris, const f184gi_light* light,
                     const float* shadow_depth, float* rgba, uint32_t* counts, int nthreads);

/* Per-voxel shadow visibility (1 lit, 0 shadowed) for a list of voxels (i,j,k triples). */
int orc_shade(const f184gi_grid_frame* frame, uint32_t shadow_res, const float* shadow_depth,
              const uint32_t* ijk, uint64_t n, uint8_t* lit);

/* Isotropic mip chain: levels packed one after another, linear, 4 values per voxel; level 0 given. */
int orc_mip_f64(double* chain, uint32_t dim, uint32_t levels, int nthreads);
int orc_mip_f32(float* chain, uint32_t dim, uint32_t levels, int nthreads);
/* 6-direction anisotropic mips: level 0 (dim^3*4) followed, for levels >= 1, by 6 direction volumes
 * (+x,-x,+y,-y,+z,-z), each dim_l^3 * 4 values. */
int orc_mip_aniso_f64(double* chain, uint32_t dim, uint32_t levels, int nthreads);

/* Cone trace one view.  chain as produced by orc_mip_*; out: 2 * w * h * 4 values
 * ([diffuse.rgb, occlusion] plane then [specular.rgb, alpha] plane).  rows [row_begin, row_end). */
int orc_trace_f64(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t anisotropic,
                  const double* chain, const float view[16], const float proj[16], uint32_t width,
                  uint32_t height, const float* depth, const uint32_t* normal, const uint16_t* roughness,
                  const f184gi_cone_params* params, double* out, uint32_t row_begin, uint32_t row_end,
                  int nthreads);
int orc_trace_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t anisotropic,
                  const float* chain, const float view[16], const float proj[16], uint32_t width,
                  uint32_t height, const float* depth, const uint32_t* normal, const uint16_t* roughness,
                  const f184gi_cone_params* params, float* out, uint32_t row_begin, uint32_t row_end,
                  int nthreads);
/* orc_trace_f32 that also totals the cone steps (counts[0]) and level samples (counts[1]) over the traced rows */
int orc_trace_count_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso,
                        const float* chain, const float view[16], const float proj[16], uint32_t W, uint32_t H,
                        const float* depth, const uint32_t* normal, const uint16_t* rough,
                        const f184gi_cone_params* params, float* out, uint32_t rb, uint32_t re, int nthreads,
                        uint64_t counts[2]);

/* One cone from `o` (L0 voxel units) along unit `dir` (for known-answer tests of the march). */
int orc_cone_f64(const double* chain, uint32_t dim, uint32_t levels, uint32_t aniso, const double o[3],
                 const double dir[3], double tan_half, const f184gi_cone_params* params, double out[4]);

/* Small restatements of reference shader helpers, exposed for known-answer tests. */
/* make_coord_space, Shader/Lighting/indirect.frag:71-86: out = x, y, z columns (9 doubles) */
void orc_make_coord_space(const double n[3], double out[9]);
/* VoxelPS packing, Pipelang/Internal/main.lua:269-270 */
uint32_t orc_pack_color565(const float rgb[3]);
uint32_t orc_pack_normal565(const float n[3]);
/* unpackColor565 / unpackNormal565, indirect.frag:88-102 */
void orc_unpack_color565(uint32_t x, double out[3]);
void orc_unpack_normal565(uint32_t x, double out[3]);
/* VoxelGS dominant axis, main.lua:100-115: 0 = Z, 1 = X, 2 = Y */
int orc_dominant_axis(const float v0[3], const float v1[3], const float v2[3]);
/* hemisphereSample_cos, Shader/math.inc:76-81 */
void orc_hemisphere_sample_cos(double u, double v, double out[3]);
/* octahedral normal codec used by the G-buffer */
uint32_t orc_oct_encode(const double n[3]);
void orc_oct_decode(uint32_t packed, double out[3]);
uint16_t orc_float_to_half(double x);
double orc_half_to_float(uint16_t h);

#ifdef __cplusplus
}
#endif

#endif
