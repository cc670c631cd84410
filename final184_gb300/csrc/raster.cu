// raster.cu -- exact, tile-binned triangle rasterizer used for the shadow map and the G-buffer.
//
// Replaces the fixed-function depth-only raster of the reference's shadow pass
// (Foreground/Renderer/ZOnlyRenderer.cpp:79-114, StaticMeshZOnlyVS Pipelang/Internal/main.lua:146-156) and the
// G-buffer pass (GBufferRenderer.cpp:79-116).  Coverage and depth are exact functions of the input:
//   clip = M * (x, y, z, 1) with M rounded to FP32, each product and sum rounded in order; a triangle inside
//   0 <= z <= w, |x|,|y| <= 16 w is divided by w (skipped for w == 1) and snapped to 1/16 pixel in FP32; any
//   other is clipped against those planes in FP64 (Sutherland-Hodgman on FP64 clip coordinates) and snapped in
//   FP64; coverage by inclusive int64 edge functions at pixel centres; depth plane z0 + a (X - X0) + b (Y - Y0)
//   solved per triangle in float-float arithmetic (clipped triangles: FP64), rounded to FP32 and evaluated in
//   FP32 in that operation order; per pixel the minimum of key = (depth bits << 32 | triangle index) wins.
// FP64 is left to clipped triangles (the FP64 pipe of GB300 is narrow: an FP64 transform and snap of every
// triangle kept it 85% busy, and the FP64 plane solve alone cost ~0.02 ms of a 500k-triangle voxelization).
// Work is binned into 16x16 pixel tiles (one CTA per tile, keys in shared memory).  Triangles spanning many
// tiles are walked by a whole warp, so no thread serialises over a screen-sized triangle.
#include "gi_device.cuh"
#include "util.cuh"

namespace f184 {
namespace {

constexpr int kTile = 16;
constexpr double kGuard = 16.0;
constexpr uint32_t kNone = 0xffffffffu;
constexpr int kBigCells = 8;     // records touching more tiles than this are binned by a warp ...
constexpr int kHugeCells = 512;  // ... or, above this many tiles, by a whole CTA
constexpr uint32_t kStage = 256;  // records staged per round by raster_tiles (one per thread)
// ceil(65536 / w) for the clipped box widths w = 1..16 of a tile: p / w = (p * c_wmagic[w]) >> 16 for p < 256
__constant__ uint32_t c_wmagic[17] = {0,    65536, 32768, 21846, 16384, 13108, 10923, 9363, 8192,
                                      7282, 6554,  5958,  5462,  5042,  4682,  4370,  4096};

// 48 bytes, 16-byte aligned: a record moves as three 16-byte loads or stores (the binning, staging and set-up
// kernels read or write whole records; 0.562 -> 0.549 ms per 500k-triangle voxelization)
struct __align__(16) SubTri {
    int32_t X[3], Y[3];
    float z0, a, b;
    uint32_t tri;
    uint16_t x0, x1, y0, y1;
};

struct V4 {
    double x, y, z, w;
};

__device__ __forceinline__ double plane_dist(int k, const V4& v) {
    switch (k) {
        case 0: return v.z;
        case 1: return dsub(v.w, v.z);
        case 2: return dsub(dmul(kGuard, v.w), v.x);
        case 3: return dadd(v.x, dmul(kGuard, v.w));
        case 4: return dsub(dmul(kGuard, v.w), v.y);
        default: return dadd(v.y, dmul(kGuard, v.w));
    }
}

__device__ int clip_polygon(V4* poly, int n) {
    V4 tmp[12];
    for (int k = 0; k < 6; ++k) {
        int m = 0;
        for (int i = 0; i < n; ++i) {
            V4 a = poly[i];
            V4 b = poly[(i + 1) % n];
            double da = plane_dist(k, a), db = plane_dist(k, b);
            bool ina = da >= 0.0, inb = db >= 0.0;
            if (ina) tmp[m++] = a;
            if (ina != inb) {
                double t = __ddiv_rn(da, dsub(da, db));
                V4 r;
                r.x = dadd(a.x, dmul(t, dsub(b.x, a.x)));
                r.y = dadd(a.y, dmul(t, dsub(b.y, a.y)));
                r.z = dadd(a.z, dmul(t, dsub(b.z, a.z)));
                r.w = dadd(a.w, dmul(t, dsub(b.w, a.w)));
                tmp[m++] = r;
            }
        }
        n = m;
        if (n < 3) return 0;
        for (int i = 0; i < n; ++i) poly[i] = tmp[i];
    }
    return n;
}

// x / w with the division skipped when w is exactly 1 (orthographic frames): x / 1 == x in IEEE arithmetic
__device__ __forceinline__ double persp_div(double x, double w) { return w == 1.0 ? x : __ddiv_rn(x, w); }

// Snapped triangle from its vertices in 1/16 pixel (X, Y) and NDC depth Z: orientation, the depth plane through
// the three (FP32 result) and the pixel range.  With zf (the depths as the FP32 values they are, for triangles
// inside the clip volume) the plane is solved in float-float arithmetic; a clipped triangle's FP64 depths are
// solved in FP64.
__device__ __forceinline__ bool snap_finish(int64_t (&X)[3], int64_t (&Y)[3], double (&Z)[3], const float* zf,
                                            uint32_t W, uint32_t H, uint32_t tri, SubTri& s) {
    float z[3] = {0.0f, 0.0f, 0.0f};
    if (zf) z[0] = zf[0], z[1] = zf[1], z[2] = zf[2];
    int64_t area2 = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
    if (area2 == 0) return false;
    if (area2 < 0) {
        int64_t t;
        t = X[1], X[1] = X[2], X[2] = t;
        t = Y[1], Y[1] = Y[2], Y[2] = t;
        double tz = Z[1];
        Z[1] = Z[2], Z[2] = tz;
        const float tzf = z[1];
        z[1] = z[2], z[2] = tzf;
        area2 = -area2;
    }
    int64_t mnx = min(X[0], min(X[1], X[2])), mxx = max(X[0], max(X[1], X[2]));
    int64_t mny = min(Y[0], min(Y[1], Y[2])), mxy = max(Y[0], max(Y[1], Y[2]));
    int64_t x0 = max(int64_t(0), -floor_div64(-(mnx - 8), 16));
    int64_t x1 = min(int64_t(W) - 1, floor_div64(mxx - 8, 16));
    int64_t y0 = max(int64_t(0), -floor_div64(-(mny - 8), 16));
    int64_t y1 = min(int64_t(H) - 1, floor_div64(mxy - 8, 16));
    if (x0 > x1 || y0 > y1) return false;
    if (zf) {
        // depth plane, float-float: dz exactly (two-sum of FP32 depths), the edge components exactly (|d| < 2^22),
        // twice the area as an exact pair (< 2^45: the remainder of its FP32 rounding is below 2^21)
        FF dz1, dz2;
        two_sum(z[1], -z[0], dz1.h, dz1.l);
        two_sum(z[2], -z[0], dz2.h, dz2.l);
        const float dx1 = float(int32_t(X[1] - X[0])), dy1 = float(int32_t(Y[1] - Y[0]));
        const float dx2 = float(int32_t(X[2] - X[0])), dy2 = float(int32_t(Y[2] - Y[0]));
        // area2 = hi 2^22 + lo with both parts exact in FP32: their two-sum is RN(area2) and its exact remainder,
        // formed without the 64-bit conversions (FP64 pipe)
        FF D;
        two_sum(__fmul_rn(float(int32_t(area2 >> 22)), 4194304.0f), float(int32_t(area2 & 0x3fffff)), D.h, D.l);
        const FF na = ff_add(ff_mul(dz1, FF{dy2, 0.0f}), ff_mul(dz2, FF{-dy1, 0.0f}));
        const FF nb = ff_add(ff_mul(dz2, FF{dx1, 0.0f}), ff_mul(dz1, FF{-dx2, 0.0f}));
        s.z0 = z[0];
        s.a = ff_div(na, D).h;
        s.b = ff_div(nb, D).h;
    } else {  // depth plane through the three snapped vertices (FP64 solve, FP32 result)
        double dx1 = double(X[1] - X[0]), dy1 = double(Y[1] - Y[0]);
        double dx2 = double(X[2] - X[0]), dy2 = double(Y[2] - Y[0]);
        double dz1 = dsub(Z[1], Z[0]), dz2 = dsub(Z[2], Z[0]);
        double D = double(area2);
        double na = dsub(dmul(dz1, dy2), dmul(dz2, dy1));
        double nb = dsub(dmul(dz2, dx1), dmul(dz1, dx2));
        s.z0 = __double2float_rn(Z[0]);
        s.a = __double2float_rn(__ddiv_rn(na, D));
        s.b = __double2float_rn(__ddiv_rn(nb, D));
    }
    for (int i = 0; i < 3; ++i) {
        s.X[i] = int32_t(X[i]);
        s.Y[i] = int32_t(Y[i]);
    }
    s.tri = tri;
    s.x0 = uint16_t(x0), s.x1 = uint16_t(x1), s.y0 = uint16_t(y0), s.y1 = uint16_t(y1);
    return true;
}

// A clipped polygon's fan triangle (FP64 clip coordinates).
__device__ bool snap(const V4& a, const V4& b, const V4& c, uint32_t W, uint32_t H, uint32_t tri, SubTri& s) {
    const V4* v[3] = {&a, &b, &c};
    int64_t X[3], Y[3];
    double Z[3];
    for (int i = 0; i < 3; ++i) {
        if (!(v[i]->w > 0.0)) return false;
        double nx = persp_div(v[i]->x, v[i]->w), ny = persp_div(v[i]->y, v[i]->w), nz = persp_div(v[i]->z, v[i]->w);
        X[i] = __double2ll_rn(dmul(dadd(nx, 1.0), 8.0 * double(W)));
        Y[i] = __double2ll_rn(dmul(dadd(ny, 1.0), 8.0 * double(H)));
        Z[i] = nz;
    }
    return snap_finish(X, Y, Z, nullptr, W, H, tri, s);
}

// The common case: a triangle inside the clip volume (0 <= z <= w, |x|, |y| <= 16 w), its clip coordinates in
// FP32 (row . (x, y, z, 1) with the FP32-rounded matrix, each product and sum rounded in order), the perspective
// division (skipped for w == 1) and the snap to 1/16 pixel in FP32; the plane in float-float.
struct V4f {
    float x, y, z, w;
};
__device__ __forceinline__ float frow(const float* r, float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r[0], x), __fmul_rn(r[1], y)), __fmul_rn(r[2], z)), r[3]);
}
__device__ __forceinline__ bool inside_f(const V4f& v) {
    const float g = __fmul_rn(16.0f, v.w);
    return v.z >= 0.0f && __fsub_rn(v.w, v.z) >= 0.0f && __fsub_rn(g, v.x) >= 0.0f && __fadd_rn(v.x, g) >= 0.0f &&
           __fsub_rn(g, v.y) >= 0.0f && __fadd_rn(v.y, g) >= 0.0f;
}
__device__ __forceinline__ float persp_div_f(float x, float w) { return w == 1.0f ? x : __fdiv_rn(x, w); }
__device__ __forceinline__ bool snap_f(const V4f (&v)[3], uint32_t W, uint32_t H, uint32_t tri, SubTri& s) {
    int64_t X[3], Y[3];
    double Z[3];
    float zf[3];
    const float sw = 8.0f * float(W), sh = 8.0f * float(H);  // exact: W, H <= 8192
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (!(v[i].w > 0.0f)) return false;
        // inside the guard band |X|, |Y| < 17 * 8 * 8192 < 2^21: the 32-bit conversion rounds the same (the
        // 64-bit one runs on the FP64 pipe)
        X[i] = __float2int_rn(__fmul_rn(__fadd_rn(persp_div_f(v[i].x, v[i].w), 1.0f), sw));
        Y[i] = __float2int_rn(__fmul_rn(__fadd_rn(persp_div_f(v[i].y, v[i].w), 1.0f), sh));
        zf[i] = persp_div_f(v[i].z, v[i].w);
        Z[i] = double(zf[i]);
    }
    return snap_finish(X, Y, Z, zf, W, H, tri, s);
}

// Edge function of (a, b) at p (1/16-pixel units): every factor fits 32 bits (snapped vertices and pixel centres
// lie within the guard band, |difference| < 2^22), so each product is one 32 x 32 -> 64-bit multiply.
__device__ __forceinline__ int64_t edge(const SubTri& s, int a, int b, int64_t px, int64_t py) {
    const int32_t dx = s.X[b] - s.X[a], dy = s.Y[b] - s.Y[a];
    const int32_t ry = int32_t(py) - s.Y[a], rx = int32_t(px) - s.X[a];
    return int64_t(dx) * int64_t(ry) - int64_t(dy) * int64_t(rx);
}

// Can the triangle cover any pixel centre of tile (tx, ty)?  Rejects tiles wholly outside one edge.
__device__ __forceinline__ bool tile_may_overlap(const SubTri& s, int tx, int ty) {
    int64_t px0 = int64_t(tx) * kTile * 16 + 8, px1 = px0 + (kTile - 1) * 16;
    int64_t py0 = int64_t(ty) * kTile * 16 + 8, py1 = py0 + (kTile - 1) * 16;
    const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
    for (int e = 0; e < 3; ++e) {
        int64_t dx = s.X[eb[e]] - s.X[ea[e]], dy = s.Y[eb[e]] - s.Y[ea[e]];
        // e(p) = dx (py - ya) - dy (px - xa): maximise over the tile corners
        int64_t px = dy > 0 ? px0 : px1;
        int64_t py = dx > 0 ? py1 : py0;
        if (edge(s, ea[e], eb[e], px, py) < 0) return false;
    }
    return true;
}

struct RasterScratch {
    SubTri* recs;          // ntris primary + overflow
    uint32_t* ovf_count;   // [1]
    uint32_t* tile_count;  // ntiles
    uint32_t* tile_start;  // ntiles
    uint32_t* tile_fill;   // ntiles
    uint32_t* total;       // [1]
    uint32_t* scan_tmp;
    uint32_t* list;
    uint32_t* big;         // records with more than kHugeCells tiles (binned by raster_bin_big, a CTA each)
    uint32_t* big_count;   // [1]
    uint32_t* mid;         // records with kBigCells < tiles <= kHugeCells (raster_bin_big, a warp each)
    uint32_t* mid_count;   // [1]
    uint64_t list_cap;
    uint64_t ovf_cap;
};

__global__ void __launch_bounds__(128) raster_setup(const float* __restrict__ tri, uint64_t ntris, RasterJob job,
                                                    RasterScratch sc, uint32_t* status) {
    const double* M = job.d_M ? job.d_M : job.M;
    __shared__ float mf[16];
    if (threadIdx.x < 16) mf[threadIdx.x] = __double2float_rn(M[threadIdx.x]);
    __syncthreads();
    uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    bool finite = true;  // a triangle with a NaN or infinite coordinate is skipped (and reported)
#pragma unroll
    for (int i = 0; i < 9; ++i) finite = finite && isfinite(tri[t * 9 + i]);
    if (!finite) {
        set_status(status, kStatusNonFinite);
        sc.recs[t].tri = kNone;
        return;
    }
    V4f cf[3];
    bool inside = true;
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const float x = tri[t * 9 + v * 3], y = tri[t * 9 + v * 3 + 1], z = tri[t * 9 + v * 3 + 2];
        cf[v] = V4f{frow(mf, x, y, z), frow(mf + 4, x, y, z), frow(mf + 8, x, y, z), frow(mf + 12, x, y, z)};
        inside = inside && inside_f(cf[v]);
    }
    if (inside) {  // one sub-triangle, the record of the triangle itself
        SubTri s;
        if (snap_f(cf, job.width, job.height, uint32_t(t), s))
            sc.recs[t] = s;
        else
            sc.recs[t].tri = kNone;
        return;
    }
    // clipped against the near/far planes or the guard band: FP64 clip coordinates and Sutherland-Hodgman
    V4 poly[12];
    for (int v = 0; v < 3; ++v) {
        const double x = tri[t * 9 + v * 3], y = tri[t * 9 + v * 3 + 1], z = tri[t * 9 + v * 3 + 2];
        poly[v] = V4{drow(M, x, y, z), drow(M + 4, x, y, z), drow(M + 8, x, y, z), drow(M + 12, x, y, z)};
    }
    const int n = clip_polygon(poly, 3);
    bool primary_done = false;
    for (int i = 1; i + 1 < n; ++i) {
        SubTri s;
        if (!snap(poly[0], poly[i], poly[i + 1], job.width, job.height, uint32_t(t), s)) continue;
        uint64_t rec;
        if (!primary_done) {
            rec = t;
            primary_done = true;
        } else {
            uint32_t k = atomicAdd(sc.ovf_count, 1u);
            if (k >= sc.ovf_cap) {
                set_status(status, kStatusOverflow);
                continue;
            }
            rec = ntris + k;
        }
        sc.recs[rec] = s;
    }
    if (!primary_done) sc.recs[t].tri = kNone;
}

__device__ __forceinline__ void bin_cell(const SubTri& s, uint32_t rec, int tx, int ty, bool test, uint32_t tiles_x,
                                         const RasterScratch& sc, uint32_t* status, bool emit) {
    if (test && !tile_may_overlap(s, tx, ty)) return;
    uint32_t t = uint32_t(ty) * tiles_x + uint32_t(tx);
    if (!emit) {
        atomicAdd(&sc.tile_count[t], 1u);
    } else {
        uint64_t slot = uint64_t(sc.tile_start[t]) + atomicAdd(&sc.tile_fill[t], 1u);
        if (slot < sc.list_cap)
            sc.list[slot] = rec;
        else
            set_status(status, kStatusOverflow);
    }
}

// Count (emit = 0) or list (emit = 1) the tiles of every record with at most kBigCells tiles; larger records are
// queued (count pass) for raster_bin_big, which gives each its own CTA.
__global__ void __launch_bounds__(128) raster_bin(uint64_t ntris, RasterScratch sc, uint32_t tiles_x, uint32_t* status,
                                                  int emit) {
    const uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t nrec = ntris + min(uint64_t(*sc.ovf_count), sc.ovf_cap);
    if (r >= nrec) return;
    const SubTri s = sc.recs[r];
    if (s.tri == kNone) return;
    const int tx0 = s.x0 / kTile, ty0 = s.y0 / kTile;
    const int ntx = s.x1 / kTile - tx0 + 1, ncell = ntx * (s.y1 / kTile - ty0 + 1);
    if (ncell > kBigCells) {
        if (!emit) {
            const bool huge = ncell > kHugeCells;
            uint32_t k = atomicAdd(huge ? sc.big_count : sc.mid_count, 1u);
            if (k < uint32_t(nrec)) (huge ? sc.big : sc.mid)[k] = uint32_t(r);
        }
        return;
    }
    for (int c = 0; c < ncell; ++c)
        bin_cell(s, uint32_t(r), tx0 + c % ntx, ty0 + c / ntx, ncell > 2, tiles_x, sc, status, emit != 0);
}

// Records of more than kHugeCells tiles take a CTA each; the others above kBigCells take a warp each, all in one
// wave (a record of a few dozen tiles would leave most of a CTA idle, and a CTA walking them one after another
// waits on each record's loads in turn).
__global__ void __launch_bounds__(256) raster_bin_big(RasterScratch sc, uint32_t tiles_x, uint32_t* status, int emit) {
    const uint32_t nbig = *sc.big_count;
    for (uint32_t i = blockIdx.x; i < nbig; i += gridDim.x) {
        const uint32_t r = sc.big[i];
        const SubTri s = sc.recs[r];
        const int tx0 = s.x0 / kTile, ty0 = s.y0 / kTile;
        const int ntx = s.x1 / kTile - tx0 + 1, ncell = ntx * (s.y1 / kTile - ty0 + 1);
        for (int c = int(threadIdx.x); c < ncell; c += int(blockDim.x))
            bin_cell(s, r, tx0 + c % ntx, ty0 + c / ntx, true, tiles_x, sc, status, emit != 0);
    }
    const uint32_t nmid = *sc.mid_count, wpb = blockDim.x / 32, lane = threadIdx.x & 31;
    for (uint32_t i = blockIdx.x * wpb + threadIdx.x / 32; i < nmid; i += gridDim.x * wpb) {
        const uint32_t r = sc.mid[i];
        const SubTri s = sc.recs[r];
        const int tx0 = s.x0 / kTile, ty0 = s.y0 / kTile;
        const int ntx = s.x1 / kTile - tx0 + 1, ncell = ntx * (s.y1 / kTile - ty0 + 1);
        for (int c = int(lane); c < ncell; c += 32)
            bin_cell(s, r, tx0 + c % ntx, ty0 + c / ntx, true, tiles_x, sc, status, emit != 0);
    }
}

// The clipped pixel box of record s in tile (tx, ty): false when empty.
__device__ __forceinline__ bool tile_box(const SubTri& s, int tx, int ty, int& x0, int& x1, int& y0, int& y1) {
    x0 = max(int(s.x0), tx * kTile), x1 = min(int(s.x1), tx * kTile + kTile - 1);
    y0 = max(int(s.y0), ty * kTile), y1 = min(int(s.y1), ty * kTile + kTile - 1);
    return x0 <= x1 && y0 <= y1;
}

// Key of record s at pixel (px, py) when its centre is covered (inclusive edges), else ~0.
__device__ __forceinline__ unsigned long long pixel_key(const SubTri& s, int px, int py, int64_t E0, int64_t E1,
                                                        int64_t E2) {
    if (E0 < 0 || E1 < 0 || E2 < 0) return ~0ull;
    // |P - X0| < 2^21: the int32 -> float conversion is exact (an int64 conversion would use the FP64 pipe)
    const int32_t dX = (16 * px + 8) - s.X[0], dY = (16 * py + 8) - s.Y[0];
    float z = __fadd_rn(__fadd_rn(s.z0, __fmul_rn(s.a, float(dX))), __fmul_rn(s.b, float(dY)));
    if (!(z > 0.0f)) z = 0.0f;  // also maps -0 and NaN to +0
    if (z > 1.0f) z = 1.0f;
    return (uint64_t(__float_as_uint(z)) << 32) | s.tri;
}

// Records whose box covers at least this many of a tile's 256 pixels are tested by every thread at its own pixel
constexpr int kWidePx = 128;

__global__ void __launch_bounds__(256) raster_tiles(RasterScratch sc, uint32_t tiles_x, uint32_t W, uint32_t H,
                                                    unsigned long long* __restrict__ keys) {
    __shared__ unsigned long long sk[kTile * kTile];
    __shared__ SubTri srec[kStage];
    __shared__ uint16_t s_wide[kStage], s_narrow[kStage];
    __shared__ uint32_t s_cnt[2][2];  // [round parity][wide, narrow]
    const uint32_t tile = blockIdx.x;
    const int tx = int(tile % tiles_x), ty = int(tile / tiles_x);
    sk[threadIdx.x] = ~0ull;
    if (threadIdx.x < 4) s_cnt[threadIdx.x >> 1][threadIdx.x & 1] = 0;
    __syncthreads();
    const uint32_t beg = sc.tile_start[tile], cnt = sc.tile_count[tile];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t end = uint32_t(min(uint64_t(beg) + cnt, sc.list_cap));
    // this thread's pixel, for the wide records
    const int mpx = tx * kTile + int(threadIdx.x % kTile), mpy = ty * kTile + int(threadIdx.x / kTile);
    unsigned long long mine = ~0ull;
    uint32_t round = 0;
    // The tile's records are staged kStage at a time, one per thread (the two dependent loads of every record in
    // flight together), and sorted by their box in the tile: a wide record (a floor under the whole map covers
    // every tile) is tested by all 256 threads at their own pixels, keeping the minimum in a register, so no
    // warp walks 256 pixels alone while the others wait at the barrier; the narrow ones are walked by the warps.
    for (uint32_t c0 = beg; c0 < end; c0 += kStage, ++round) {
        const uint32_t n = min(end - c0, uint32_t(kStage));
        uint32_t* cnts = s_cnt[round & 1];
        if (threadIdx.x < n) {
            const SubTri s = sc.recs[sc.list[c0 + threadIdx.x]];
            srec[threadIdx.x] = s;
            int x0, x1, y0, y1;
            if (tile_box(s, tx, ty, x0, x1, y0, y1)) {
                if ((x1 - x0 + 1) * (y1 - y0 + 1) >= kWidePx)
                    s_wide[atomicAdd(&cnts[0], 1u)] = uint16_t(threadIdx.x);
                else
                    s_narrow[atomicAdd(&cnts[1], 1u)] = uint16_t(threadIdx.x);
            }
        }
        __syncthreads();
        const uint32_t nwide = cnts[0], nnarrow = cnts[1];
        if (threadIdx.x < 2) s_cnt[(round + 1) & 1][threadIdx.x] = 0;  // the next round's counters
        for (uint32_t k = 0; k < nwide; ++k) {
            const SubTri& s = srec[s_wide[k]];
            const int64_t Px = int64_t(mpx) * 16 + 8, Py = int64_t(mpy) * 16 + 8;
            const unsigned long long key = pixel_key(s, mpx, mpy, edge(s, 1, 2, Px, Py), edge(s, 2, 0, Px, Py),
                                                     edge(s, 0, 1, Px, Py));
            mine = key < mine ? key : mine;
        }
        // Each warp rasterizes GROUPS narrow records at once, LANES lanes per record: the per-record set-up
        // (clipping, the edge functions at the box corner, the row divisor) is spread over the warp's lanes
        // instead of being repeated by all 32 for one record, and the record's pixels are walked LANES at a time.
        constexpr uint32_t GROUPS = 4, LANES = 32 / GROUPS;
        const uint32_t grp = lane / LANES, sub = lane % LANES;
        for (uint32_t r0 = warp * GROUPS; r0 < nnarrow; r0 += 8 * GROUPS) {
            const uint32_t r = r0 + grp;
            if (r >= nnarrow) continue;
            const SubTri& s = srec[s_narrow[r]];
            int x0, x1, y0, y1;
            tile_box(s, tx, ty, x0, x1, y0, y1);
            const int w = x1 - x0 + 1, npx = w * (y1 - y0 + 1);
            // Edge functions at the box's first pixel centre (int64), stepped exactly in int32 within the tile:
            // |edge delta| < 2^21 and the offsets are below 16 pixels (256 units), so each step term is < 2^29.
            const int64_t Px0 = int64_t(x0) * 16 + 8, Py0 = int64_t(y0) * 16 + 8;
            const int64_t E0 = edge(s, 1, 2, Px0, Py0), E1 = edge(s, 2, 0, Px0, Py0), E2 = edge(s, 0, 1, Px0, Py0);
            const int32_t ax0 = s.X[2] - s.X[1], ay0 = s.Y[2] - s.Y[1], ax1 = s.X[0] - s.X[2], ay1 = s.Y[0] - s.Y[2],
                          ax2 = s.X[1] - s.X[0], ay2 = s.Y[1] - s.Y[0];
            const uint32_t wmagic = c_wmagic[w];  // p / w = (p * wmagic) >> 16, p < 256
            for (int p = int(sub); p < npx; p += int(LANES)) {
                const int ly = int((uint32_t(p) * wmagic) >> 16), lx = p - ly * w;
                const int px = x0 + lx, py = y0 + ly;
                const int32_t ox = 16 * lx, oy = 16 * ly;
                const unsigned long long key =
                    pixel_key(s, px, py, E0 + int64_t(ax0 * oy - ay0 * ox), E1 + int64_t(ax1 * oy - ay1 * ox),
                              E2 + int64_t(ax2 * oy - ay2 * ox));
                if (key != ~0ull) atomicMin(&sk[(py - ty * kTile) * kTile + (px - tx * kTile)], key);
            }
        }
        __syncthreads();  // srec is restaged for the next records
    }
    if (mpx < int(W) && mpy < int(H)) {
        const unsigned long long k = sk[threadIdx.x];
        keys[uint64_t(mpy) * W + mpx] = k < mine ? k : mine;
    }
}

template <class T>
T* carve(char*& p, uint64_t n) {
    uintptr_t a = (reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255);
    T* r = reinterpret_cast<T*>(a);
    p = reinterpret_cast<char*>(a + n * sizeof(T));
    return r;
}

}  // namespace

static uint64_t ovf_capacity(uint64_t ntris) { return ntris / 2 + 4096; }
static constexpr uint32_t kBigBlocks = 8 * 152;
static uint64_t list_capacity(uint64_t ntris, uint32_t ntiles) { return ntris * 8 + uint64_t(ntiles) * 16 + 65536; }

size_t raster_scratch_bytes(uint64_t ntris, uint32_t W, uint32_t H) {
    uint32_t tiles = ((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    uint64_t recs = ntris + ovf_capacity(ntris);
    return recs * sizeof(SubTri) + uint64_t(tiles) * 12 + scan_scratch_bytes(tiles) + list_capacity(ntris, tiles) * 4 +
           2 * recs * 4 + 22 * 256;
}

int raster_launch(const RasterJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status, cudaStream_t s) {
    if (job.width == 0 || job.height == 0 || job.width > kMaxRasterSide || job.height > kMaxRasterSide)
        return fail(F184GI_ERR_INVALID, "raster: viewport out of range");
    if (job.ntris >= 0xffff0000ull) return fail(F184GI_ERR_INVALID, "raster: too many triangles");
    const uint32_t tiles_x = (job.width + kTile - 1) / kTile, tiles_y = (job.height + kTile - 1) / kTile;
    const uint32_t ntiles = tiles_x * tiles_y;
    if (scratch_bytes < raster_scratch_bytes(job.ntris, job.width, job.height))
        return fail(F184GI_ERR_INVALID, "raster: scratch too small");
    char* p = static_cast<char*>(scratch);
    RasterScratch sc;
    sc.ovf_cap = ovf_capacity(job.ntris);
    sc.recs = carve<SubTri>(p, job.ntris + sc.ovf_cap);
    sc.ovf_count = carve<uint32_t>(p, 1);
    sc.total = carve<uint32_t>(p, 1);
    sc.tile_count = carve<uint32_t>(p, ntiles);
    sc.tile_start = carve<uint32_t>(p, ntiles);
    sc.tile_fill = carve<uint32_t>(p, ntiles);
    sc.scan_tmp = carve<uint32_t>(p, scan_scratch_bytes(ntiles) / 4);
    sc.list_cap = list_capacity(job.ntris, ntiles);
    sc.list = carve<uint32_t>(p, sc.list_cap);
    sc.big = carve<uint32_t>(p, job.ntris + sc.ovf_cap);
    sc.big_count = carve<uint32_t>(p, 1);
    sc.mid = carve<uint32_t>(p, job.ntris + sc.ovf_cap);
    sc.mid_count = carve<uint32_t>(p, 1);
    cudaMemsetAsync(sc.big_count, 0, 4, s);
    cudaMemsetAsync(sc.mid_count, 0, 4, s);
    cudaMemsetAsync(sc.ovf_count, 0, 4, s);
    cudaMemsetAsync(sc.tile_count, 0, size_t(ntiles) * 4, s);
    cudaMemsetAsync(sc.tile_fill, 0, size_t(ntiles) * 4, s);
    const uint64_t nrec = job.ntris + sc.ovf_cap;
    const uint32_t bin_blocks = uint32_t((nrec + 127) / 128);
    if (job.ntris) {
        raster_setup<<<uint32_t((job.ntris + 127) / 128), 128, 0, s>>>(job.tri, job.ntris, job, sc, d_status);
        raster_bin<<<bin_blocks, 128, 0, s>>>(job.ntris, sc, tiles_x, d_status, 0);
        raster_bin_big<<<kBigBlocks, 256, 0, s>>>(sc, tiles_x, d_status, 0);
        note_launches(3);
    }
    int rc = exclusive_scan(sc.tile_count, ntiles, sc.tile_start, sc.total, sc.scan_tmp, s);
    if (rc) return rc;
    if (job.ntris) {
        raster_bin<<<bin_blocks, 128, 0, s>>>(job.ntris, sc, tiles_x, d_status, 1);
        raster_bin_big<<<kBigBlocks, 256, 0, s>>>(sc, tiles_x, d_status, 1);
        note_launches(2);
    }
    raster_tiles<<<ntiles, 256, 0, s>>>(sc, tiles_x, job.width, job.height, job.keys);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "raster");
}

// ---------------- G-buffer resolve ----------------
namespace {

__device__ __forceinline__ uint32_t oct_encode(float3 n) {
    float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    float x = n.x / s, y = n.y / s;
    if (n.z < 0.0f) {
        float ox = x, oy = y;
        x = (1.0f - fabsf(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
        y = (1.0f - fabsf(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
    }
    return uint32_t(__half_as_ushort(__float2half_rn(x))) | (uint32_t(__half_as_ushort(__float2half_rn(y))) << 16);
}

struct Mat3x4 {
    float m[12];
};

__global__ void gbuffer_resolve(const unsigned long long* __restrict__ keys, uint32_t W, uint32_t H,
                                const float* __restrict__ tri, const float* __restrict__ rough, Mat3x4 V, float3 eye,
                                float* depth, uint32_t* normal, uint16_t* rough_out, uint32_t* tri_out) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= uint64_t(W) * H) return;
    unsigned long long k = keys[i];
    if (k == ~0ull) {
        depth[i] = 1.0f;
        normal[i] = 0;
        rough_out[i] = 0;
        if (tri_out) tri_out[i] = 0xffffffffu;
        return;
    }
    uint32_t t = uint32_t(k & 0xffffffffu);
    depth[i] = __uint_as_float(uint32_t(k >> 32));
    const float* p = tri + uint64_t(t) * 9;
    float3 p0 = make_float3(p[0], p[1], p[2]), p1 = make_float3(p[3], p[4], p[5]), p2 = make_float3(p[6], p[7], p[8]);
    float3 a = make_float3(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z), b = make_float3(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z);
    float3 n = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
    float il = rsqrtf(fmaxf(n.x * n.x + n.y * n.y + n.z * n.z, 1e-30f));
    n = make_float3(n.x * il, n.y * il, n.z * il);
    if (n.x * (eye.x - p0.x) + n.y * (eye.y - p0.y) + n.z * (eye.z - p0.z) < 0.0f) n = make_float3(-n.x, -n.y, -n.z);
    float3 nv = make_float3(V.m[0] * n.x + V.m[1] * n.y + V.m[2] * n.z, V.m[4] * n.x + V.m[5] * n.y + V.m[6] * n.z,
                            V.m[8] * n.x + V.m[9] * n.y + V.m[10] * n.z);
    float nl = rsqrtf(fmaxf(nv.x * nv.x + nv.y * nv.y + nv.z * nv.z, 1e-30f));
    nv = make_float3(nv.x * nl, nv.y * nl, nv.z * nl);
    normal[i] = oct_encode(nv);
    rough_out[i] = __half_as_ushort(__float2half_rn(rough[t]));
    if (tri_out) tri_out[i] = t;
}

}  // namespace

int gbuffer_resolve_launch(const unsigned long long* keys, uint32_t W, uint32_t H, const float* tri,
                           const float* rough, const float view[16], const float eye[3], float* depth,
                           uint32_t* normal, uint16_t* rough_out, uint32_t* tri_out, cudaStream_t s) {
    Mat3x4 V;
    for (int i = 0; i < 12; ++i) V.m[i] = view[i];
    uint64_t n = uint64_t(W) * H;
    gbuffer_resolve<<<uint32_t((n + 255) / 256), 256, 0, s>>>(keys, W, H, tri, rough, V,
                                                              make_float3(eye[0], eye[1], eye[2]), depth, normal,
                                                              rough_out, tri_out);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "gbuffer_resolve");
}

}  // namespace f184
