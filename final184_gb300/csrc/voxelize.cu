// voxelize.cu -- conservative voxelization with shadow-mapped direct-light injection into 8^3 bricks.
//
// Replaces the reference's VoxelGS/VoxelPS pair (Pipelang/Internal/main.lua:83-144, 242-275), which projects
// each triangle on its dominant axis and stores an RGB565 albedo + normal per covered pixel centre with
// last-writer-wins imageStore.  Here a voxel is covered when the triangle and the closed voxel box overlap
// (separating-axis test), decided exactly in integers on vertices snapped to 1/256 voxel (FP64 snap).  Each
// covering triangle adds its Lambert weight |dot(-L, n)| * albedo (the term of Shader/Lighting/indirect.frag:60-62,
// 167) as 1.31 fixed point with 64-bit integer atomics, so sums and counts are independent of triangle order.  The
// voxel's radiance is luminance * shadow(voxel centre) * mean weight, the shadow test being indirect.frag:160-165's
// compare with a two-voxel bias, evaluated as a fixed FP32 operation sequence (the same decision on any IEEE
// machine) against the shadow map rasterized by raster.cu.  FP64 is used per vertex only (the snap).
//
// Pipeline: setup (snap, weight, count overlapped bricks) -> scan -> emit (triangle lists per brick) -> items
// (each (triangle, brick) pair's exact-test setup) -> one CTA per brick accumulates in shared memory, resolves and
// writes the brick once.
#include "gi_device.cuh"
#include "util.cuh"

namespace f184 {
namespace {

constexpr int64_t kFix = 256;     // fixed-point units per voxel
constexpr int64_t kHalf = 128;
constexpr int64_t kBrickFix = 2048;  // units per brick edge
constexpr int64_t kMaxQ = int64_t(1) << 19;
constexpr uint32_t kInvalid = 0xffffffffu;

__constant__ float c_albedo_lut[256];  // (i / 255)^2.2

// 16-byte aligned (48 bytes): a record moves as three 16-byte loads or stores
struct __align__(16) TriRec {
    int32_t q[9];    // snapped vertices (x0 y0 z0 x1 ...), 24.8 voxel fixed point
    uint32_t wq[3];  // injection weight per channel, 1.31 fixed point (<= 2^31); wq[0] = kInvalid marks skipped
};

struct ItemSetup;

struct VoxScratch {
    TriRec* recs;
    uint32_t* brick_count;
    uint32_t* brick_start;
    uint32_t* brick_fill;
    uint32_t* total;
    uint32_t* scan_tmp;
    uint32_t* dirty_mask;  // nbricks bits, null = all bricks
    uint32_t* list;        // triangle of each (triangle, brick) item, grouped by brick
    uint32_t* list_brick;  // brick of each item
    ItemSetup* items;      // each item's exact-test setup (vox_items), in list order
    uint32_t* big;        // triangles with more than kMidCells bricks (binned by vox_bin_big, a CTA each)
    uint32_t* big_count;  // [1]
    uint32_t* mid;        // triangles with kThreadCells < bricks <= kMidCells (vox_bin_big, a warp each)
    uint32_t* mid_count;  // [1]
    uint2* mid_bits;      // per mid entry: which of its (up to 64) bricks the count pass listed
    uint8_t* bits;        // per triangle of at most kThreadCells bricks: which of them the count pass listed
    uint64_t list_cap;
};

__device__ __forceinline__ int64_t iabs64(int64_t x) { return x < 0 ? -x : x; }
__device__ __forceinline__ int64_t sar7_floor(int64_t x) { return x >> 7; }         // floor(x / 128)
__device__ __forceinline__ int64_t sar7_ceil(int64_t x) { return -((-x) >> 7); }    // ceil(x / 128)
__device__ __forceinline__ int32_t clamp32(int64_t x) {
    return int32_t(x > int64_t(INT32_MAX) ? int64_t(INT32_MAX) : (x < int64_t(INT32_MIN) ? int64_t(INT32_MIN) : x));
}

// The nine edge x unit-axis tests of a triangle (box-relative vertices v) against the box of half size h.
template <class T>
__device__ __forceinline__ bool sat_edges(const T (&v)[3][3], T h) {
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        T ed[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) ed[b] = v[(e + 1) % 3][b] - v[e][b];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            T a0 = 0, a1 = 0, a2 = 0;
            if (ax == 0) a1 = ed[2], a2 = -ed[1];
            if (ax == 1) a0 = -ed[2], a2 = ed[0];
            if (ax == 2) a0 = ed[1], a1 = -ed[0];
            const T p0 = a0 * v[0][0] + a1 * v[0][1] + a2 * v[0][2];
            const T p1 = a0 * v[1][0] + a1 * v[1][1] + a2 * v[1][2];
            const T p2 = a0 * v[2][0] + a1 * v[2][1] + a2 * v[2][2];
            const T rr = h * ((a0 < 0 ? -a0 : a0) + (a1 < 0 ? -a1 : a1) + (a2 < 0 ? -a2 : a2));
            if (min(p0, min(p1, p2)) > rr || max(p0, max(p1, p2)) < -rr) return false;
        }
    }
    return true;
}

// Exact closed-set overlap of a triangle (fixed-point q) with the axis-aligned box of centre c, half size h.
__device__ bool tri_box_sat(const int32_t* q, const int64_t c[3], int64_t h) {
    int64_t v[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) v[a][b] = int64_t(q[a * 3 + b]) - c[b];
    for (int b = 0; b < 3; ++b) {
        int64_t mn = min(v[0][b], min(v[1][b], v[2][b])), mx = max(v[0][b], max(v[1][b], v[2][b]));
        if (mn > h || mx < -h) return false;
    }
    int64_t e0[3], e1[3];
    for (int b = 0; b < 3; ++b) {
        e0[b] = v[1][b] - v[0][b];
        e1[b] = v[2][b] - v[0][b];
    }
    int64_t n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    int64_t s = n[0] * v[0][0] + n[1] * v[0][1] + n[2] * v[0][2];
    int64_t r = h * (iabs64(n[0]) + iabs64(n[1]) + iabs64(n[2]));
    if (s > r || s < -r) return false;
    // Vertices within 2^14 of the box centre (a triangle near its box: all but the largest) take the nine edge-axis
    // tests in 32-bit integers: edge components < 2^15, each product < 2^29, a projection (two nonzero terms) < 2^30,
    // the radius h (|a| + |a|) < 2^26 for h <= 2^10, so the bounds are the same integers the 64-bit form computes.
    int64_t vmax = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) vmax = max(vmax, iabs64(v[a][b]));
    if (vmax < (int64_t(1) << 14) && h <= 1024) {
        int32_t w[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) w[a][b] = int32_t(v[a][b]);
        return sat_edges<int32_t>(w, int32_t(h));
    }
    return sat_edges<int64_t>(v, h);
}

// voxel range touched by the triangle's AABB (closed boxes), clamped to the grid
__device__ __forceinline__ void voxel_range(const int32_t* q, uint32_t dim, int32_t lo[3], int32_t hi[3]) {
    for (int a = 0; a < 3; ++a) {
        int64_t mn = min(q[a], min(q[3 + a], q[6 + a])), mx = max(q[a], max(q[3 + a], q[6 + a]));
        lo[a] = int32_t(max(int64_t(0), -floor_div64(-(mn - kFix), kFix)));
        hi[a] = int32_t(min(int64_t(dim) - 1, floor_div64(mx, kFix)));
    }
}

constexpr int kThreadCells = 8;  // triangles overlapping at most this many bricks are binned by one thread,
constexpr int kMidCells = 64;    // at most this many by a warp, more by a whole CTA

// Is brick (bx, by, bz) listed for the triangle: inside the dirty set and (test) overlapped by the triangle?
__device__ __forceinline__ bool brick_hit(const int32_t* q, int bx, int by, int bz, bool test, const VoxScratch& sc) {
    const uint32_t m = morton3(bx, by, bz);
    if (sc.dirty_mask && !((sc.dirty_mask[m >> 5] >> (m & 31)) & 1u)) return false;
    if (!test) return true;
    const int64_t c[3] = {bx * kBrickFix + kBrickFix / 2, by * kBrickFix + kBrickFix / 2, bz * kBrickFix + kBrickFix / 2};
    return tri_box_sat(q, c, kBrickFix / 2);
}

// Count (emit = false) or list (emit = true) triangle t in brick m.
__device__ __forceinline__ void brick_add(uint32_t t, uint32_t m, const VoxScratch& sc, uint32_t* status, bool emit) {
    if (!emit) {
        atomicAdd(&sc.brick_count[m], 1u);
    } else {
        uint64_t slot = uint64_t(sc.brick_start[m]) + atomicAdd(&sc.brick_fill[m], 1u);
        if (slot < sc.list_cap) {
            sc.list[slot] = t;
            sc.list_brick[slot] = m;
        } else
            set_status(status, kStatusOverflow);
    }
}

__device__ __forceinline__ void bin_brick(const int32_t* q, uint32_t t, int bx, int by, int bz, bool test,
                                          const VoxScratch& sc, uint32_t* status, bool emit) {
    if (brick_hit(q, bx, by, bz, test, sc)) brick_add(t, morton3(bx, by, bz), sc, status, emit);
}

// brick box of a triangle: first brick and extent per axis
__device__ __forceinline__ int brick_box(const int32_t* q, uint32_t dim, int32_t b0[3], int32_t nb[3]) {
    int32_t lo[3], hi[3];
    voxel_range(q, dim, lo, hi);
    for (int a = 0; a < 3; ++a) b0[a] = lo[a] >> 3, nb[a] = (hi[a] >> 3) - b0[a] + 1;
    return nb[0] * nb[1] * nb[2];
}

// Count (emit = false) or list (emit = true) the bricks of a triangle with at most kThreadCells bricks; larger
// triangles are queued on the count pass and binned by vox_bin_big.  The count pass keeps which bricks it listed
// (one bit each), so the list pass repeats none of the overlap tests.
__device__ __forceinline__ void bin_small(const TriRec& r, uint32_t t, uint32_t dim, const VoxScratch& sc,
                                          uint32_t* status, bool emit, uint64_t ntris) {
    int32_t b0[3], nb[3];
    const int ncell = brick_box(r.q, dim, b0, nb);
    if (ncell > kThreadCells) {
        if (!emit) {
            const bool huge = ncell > kMidCells;
            uint32_t k = atomicAdd(huge ? sc.big_count : sc.mid_count, 1u);
            if (k < ntris) (huge ? sc.big : sc.mid)[k] = t;
        }
        return;
    }
    uint32_t bits = emit ? sc.bits[t] : 0u;
    for (int c = 0; c < ncell; ++c) {
        const int bx = b0[0] + c % nb[0], by = b0[1] + (c / nb[0]) % nb[1], bz = b0[2] + c / (nb[0] * nb[1]);
        if (emit) {
            if ((bits >> c) & 1u) brick_add(t, morton3(bx, by, bz), sc, status, true);
        } else if (brick_hit(r.q, bx, by, bz, ncell > 1, sc)) {
            brick_add(t, morton3(bx, by, bz), sc, status, false);
            bits |= 1u << c;
        }
    }
    if (!emit) sc.bits[t] = uint8_t(bits);
}

// Triangles of more than kMidCells bricks take a CTA each; the others above kThreadCells take a warp each, all in
// one wave (a CTA walking triangles of a few dozen bricks one after another would wait on each one's loads and
// overlap tests in turn with most of its threads idle).  A warp's count pass keeps its triangle's listed bricks
// as two 32-bit ballots for the list pass.
__global__ void __launch_bounds__(256) vox_bin_big(uint32_t dim, VoxScratch sc, uint32_t* status, int emit) {
    const uint32_t nbig = *sc.big_count;
    for (uint32_t i = blockIdx.x; i < nbig; i += gridDim.x) {
        const uint32_t t = sc.big[i];
        const TriRec r = sc.recs[t];
        int32_t b0[3], nb[3];
        const int n = brick_box(r.q, dim, b0, nb);
        for (int c = int(threadIdx.x); c < n; c += int(blockDim.x))
            bin_brick(r.q, t, b0[0] + c % nb[0], b0[1] + (c / nb[0]) % nb[1], b0[2] + c / (nb[0] * nb[1]), true, sc,
                      status, emit != 0);
    }
    const uint32_t nmid = *sc.mid_count, wpb = blockDim.x / 32, lane = threadIdx.x & 31;
    for (uint32_t i = blockIdx.x * wpb + threadIdx.x / 32; i < nmid; i += gridDim.x * wpb) {  // warp-uniform
        const uint32_t t = sc.mid[i];
        const TriRec r = sc.recs[t];
        int32_t b0[3], nb[3];
        const int n = brick_box(r.q, dim, b0, nb);
        const uint2 listed = emit ? sc.mid_bits[i] : make_uint2(0u, 0u);
        bool hit[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = int(lane) + 32 * h;
            const int bx = b0[0] + c % nb[0], by = b0[1] + (c / nb[0]) % nb[1], bz = b0[2] + c / (nb[0] * nb[1]);
            hit[h] = c < n && (emit ? (((h ? listed.y : listed.x) >> lane) & 1u) != 0u : brick_hit(r.q, bx, by, bz, true, sc));
            if (hit[h]) brick_add(t, morton3(bx, by, bz), sc, status, emit != 0);
        }
        const uint32_t b0bits = __ballot_sync(0xffffffffu, hit[0]), b1bits = __ballot_sync(0xffffffffu, hit[1]);
        if (!emit && lane == 0) sc.mid_bits[i] = make_uint2(b0bits, b1bits);
    }
}

__global__ void __launch_bounds__(128) vox_setup(const float* __restrict__ tri, const uint32_t* __restrict__ albedo,
                                                 uint64_t ntris, const f184gi_grid_frame* __restrict__ fr, uint32_t dim,
                                                 VoxScratch sc, uint32_t* status) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    TriRec r;
    bool ok = t < ntris;
    const float* p = tri + (ok ? t : 0) * 9;
    if (ok) {  // a triangle with a NaN or infinite coordinate is skipped (and reported)
        bool finite = true;
        for (int i = 0; i < 9; ++i) finite = finite && isfinite(p[i]);
        if (!finite) {
            set_status(status, kStatusNonFinite);
            ok = false;
        }
    }
    for (int i = 0; i < 9; ++i) {
        int a = i % 3;
        int64_t q = 0;
        if (ok) {
            double d = dsub(double(p[i]), fr->origin[a]);
            double s = dmul(d, fr->inv_voxel_fixed);
            q = __double2ll_rn(s);
        }
        if (q >= kMaxQ || q <= -kMaxQ) {
            set_status(status, kStatusRange);
            ok = false;
            q = 0;
        }
        r.q[i] = int32_t(q);
    }
    if (ok) {
        int64_t e0[3], e1[3];
        for (int a = 0; a < 3; ++a) {
            e0[a] = int64_t(r.q[3 + a]) - r.q[a];
            e1[a] = int64_t(r.q[6 + a]) - r.q[a];
        }
        int64_t n0 = e0[1] * e1[2] - e0[2] * e1[1], n1 = e0[2] * e1[0] - e0[0] * e1[2],
                n2 = e0[0] * e1[1] - e0[1] * e1[0];
        if (n0 == 0 && n1 == 0 && n2 == 0) ok = false;
        int32_t lo[3], hi[3];
        voxel_range(r.q, dim, lo, hi);
        if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) ok = false;
    }
    r.wq[0] = r.wq[1] = r.wq[2] = kInvalid;
    if (ok) {
        // injection weight |dot(-L, n)| * albedo, FP32
        float3 a = make_float3(p[3] - p[0], p[4] - p[1], p[5] - p[2]);
        float3 b = make_float3(p[6] - p[0], p[7] - p[1], p[8] - p[2]);
        float3 n = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
        const float nn = n.x * n.x + n.y * n.y + n.z * n.z;
        float wi0 = -float(fr->light_dir[0]), wi1 = -float(fr->light_dir[1]), wi2 = -float(fr->light_dir[2]);
        float cosv;
        if (nn >= 0x1p-20f * (a.x * a.x + a.y * a.y + a.z * a.z) * (b.x * b.x + b.y * b.y + b.z * b.z)) {
            // the edges are more than ~0.06 degrees apart: the FP32 normal's direction is good to ~1e-4
            const float len = sqrtf(nn);
            cosv = len > 0.0f ? fabsf(wi0 * n.x + wi1 * n.y + wi2 * n.z) / len : 0.0f;
        } else {
            // a sliver: its FP32 cross product is mostly rounding, so the normal is formed in FP64 from the
            // FP32 positions (the oracle's sequence: edge differences, cross, |n|, |dot(-L, n)| / |n|)
            const double ax = dsub(p[3], p[0]), ay = dsub(p[4], p[1]), az = dsub(p[5], p[2]);
            const double bx = dsub(p[6], p[0]), by = dsub(p[7], p[1]), bz = dsub(p[8], p[2]);
            const double nx = dsub(dmul(ay, bz), dmul(az, by)), ny = dsub(dmul(az, bx), dmul(ax, bz)),
                         nz = dsub(dmul(ax, by), dmul(ay, bx));
            const double len = __dsqrt_rn(dadd(dadd(dmul(nx, nx), dmul(ny, ny)), dmul(nz, nz)));
            const double d = dadd(dadd(dmul(-fr->light_dir[0], nx), dmul(-fr->light_dir[1], ny)),
                                  dmul(-fr->light_dir[2], nz));
            cosv = len > 0.0 ? float(__ddiv_rn(fabs(d), len)) : 0.0f;
        }
        uint32_t al = albedo[t];
        for (int c = 0; c < 3; ++c) {
            float w = cosv * c_albedo_lut[(al >> (8 * c)) & 255u];
            r.wq[c] = min(__float2uint_rn(w * 2147483648.0f), 0x80000000u);
        }
    }
    if (t < ntris) sc.recs[t] = r;
    if (ok) bin_small(r, uint32_t(t), dim, sc, status, false, ntris);
}

__global__ void __launch_bounds__(128) vox_emit(uint64_t ntris, uint32_t dim, VoxScratch sc, uint32_t* status) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const TriRec r = sc.recs[t];
    if (r.wq[0] != kInvalid) bin_small(r, uint32_t(t), dim, sc, status, true, ntris);
}

__global__ void vox_dirty_mask(const uint32_t* dirty, uint32_t ndirty, uint32_t nbricks, uint32_t* mask) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ndirty && dirty[i] < nbricks) atomicOr(&mask[dirty[i] >> 5], 1u << (dirty[i] & 31));
}

// Shadow visibility of the centre of voxel (i, j, k): the exact FP32 operation sequence of the frame's affine
// voxel -> light-clip map, nearest texel, lit iff z - bias <= stored depth (empty texels hold depth 1).
__device__ __forceinline__ bool voxel_lit(const f184gi_grid_frame* __restrict__ fr,
                                          const unsigned long long* __restrict__ shadow, uint32_t res, int i, int j,
                                          int k) {
    const float* lv = fr->light_vox;
    const float fi = float(i), fj = float(j), fk = float(k);
    float v[3];
#pragma unroll
    for (int rr = 0; rr < 3; ++rr) {
        const float* c = lv + 4 * rr;
        float s = __fadd_rn(c[0], __fmul_rn(fi, c[1]));
        s = __fadd_rn(s, __fmul_rn(fj, c[2]));
        v[rr] = __fadd_rn(s, __fmul_rn(fk, c[3]));
    }
    const float half_res = 0.5f * float(res);
    const float tx = floorf(__fmul_rn(__fadd_rn(v[0], 1.0f), half_res));
    const float ty = floorf(__fmul_rn(__fadd_rn(v[1], 1.0f), half_res));
    if (!(tx >= 0.0f && ty >= 0.0f && tx < float(res) && ty < float(res))) return true;
    const unsigned long long key = shadow[uint64_t(ty) * res + uint64_t(tx)];
    const float sd = key == ~0ull ? 1.0f : __uint_as_float(uint32_t(key >> 32));
    return __fsub_rn(v[2], fr->shadow_bias_f) <= sd;
}

// Relight: L0 radiance = luminance * (lit ? weight : 0) for every voxel of the mean-weight grid W (same brick
// layout as L0).  With vox_bricks writing W, this gives the same bytes as the fused pass; the served path runs it
// after every shadow-map change without re-voxelizing.
__global__ void __launch_bounds__(256) relight_bricks(const float4* __restrict__ W, const f184gi_grid_frame* __restrict__ fr,
                                                      uint32_t dim, ChainLayout chain, f184gi_light light,
                                                      const unsigned long long* __restrict__ shadow, uint32_t res) {
    const uint32_t nb = dim >> 3;
    const uint64_t nvox = uint64_t(nb) * nb * nb * 512;
    for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nvox; e += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t m = uint32_t(e >> 9), li = uint32_t(e & 511);
        const float4 w = W[e];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (w.w != 0.0f) {
            const int i = int(compact1by2(m)) * 8 + int(li & 7), j = int(compact1by2(m >> 1)) * 8 + int((li >> 3) & 7),
                      k = int(compact1by2(m >> 2)) * 8 + int(li >> 6);
            const bool lit = voxel_lit(fr, shadow, res, i, j, k);
            out = make_float4(light.luminance[0] * (lit ? w.x : 0.0f), light.luminance[1] * (lit ? w.y : 0.0f),
                              light.luminance[2] * (lit ? w.z : 0.0f), 1.0f);
        }
        store_vox(chain.base, chain.format, chain.off[0] + e, out);
    }
}

// Exact tests of one (triangle, brick) item, prepared by 1, 2 or 4 threads and shared through shared memory.  With
// m = 2 (voxel - brick origin) + 1 (odd, 1..15) the voxel centre is 128 m + brick offset and every separating-axis
// test reads lo <= a . m <= hi in integers.  The nine edge x unit-axis tests each ignore one coordinate, so they
// are evaluated once per cell of the three 8x8 projections of the item's voxel box into bit masks; a voxel is
// covered when its three projection bits are set and the plane test passes.
// 16-byte aligned (96 bytes with the padding): a row reads its fields with 16-byte loads
struct __align__(16) ItemSetup {
    unsigned long long mask[3];  // P = 0: bit y + 8z; P = 1: bit z + 8x; P = 2: bit x + 8y
    long long n[3];              // triangle normal (relative to the brick)
    long long plo, phi;          // plane test bounds on n . m
    uint32_t wq[3];
    uint8_t l0[3], ext[3];       // voxel box inside the brick: first voxel and extent per axis
    uint8_t small;               // |n| < 2^25 per component: the plane test of a voxel fits 32 bits
};

// The three projections' cell masks of an item (edge x unit-axis separating-axis tests), in integers of type T.
template <class T>
__device__ __forceinline__ T ceil_div128(T x) { return -((-x) >> 7); }
template <class T>
__device__ __forceinline__ void item_masks(const int32_t (&v)[3][3], const int32_t l0[3], const int32_t l1[3],
                                           int part, int per, unsigned long long (&mks)[3]) {
#pragma unroll
    for (int P = 0; P < 3; ++P) {
        unsigned long long mk = 0ull;
        // the three edge axes of projection P: a = edge x unit(P); components on the two kept axes
        const int ku = (P + 1) % 3, kw = (P + 2) % 3;  // kept axes: u first, w second
        int32_t cu[3], cw[3], lo[3], hi[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            int32_t ed[3];
#pragma unroll
            for (int b = 0; b < 3; ++b) ed[b] = v[(e + 1) % 3][b] - v[e][b];
            int32_t a[3] = {0, 0, 0};
            if (P == 0) a[1] = ed[2], a[2] = -ed[1];
            if (P == 1) a[0] = -ed[2], a[2] = ed[0];
            if (P == 2) a[0] = ed[1], a[1] = -ed[0];
            auto dotw = [&](const int32_t (&x)[3]) { return T(a[0]) * x[0] + T(a[1]) * x[1] + T(a[2]) * x[2]; };
            const T p0 = dotw(v[0]), p1 = dotw(v[1]), p2 = dotw(v[2]);
            const T rr = T(kHalf) * (T(abs(a[0])) + abs(a[1]) + abs(a[2]));
            const T pmin = min(p0, min(p1, p2)), pmax = max(p0, max(p1, p2));
            cu[e] = a[ku];
            cw[e] = a[kw];
            lo[e] = clamp32(int64_t(ceil_div128<T>(pmin - rr)));
            hi[e] = clamp32(int64_t((pmax + rr) >> 7));
        }
        for (int w = l0[kw] + part; w <= l1[kw]; w += per) {  // this thread's share of the rows
            const int32_t mw = 2 * w + 1;
            for (int u = l0[ku]; u <= l1[ku]; ++u) {
                const int32_t mu = 2 * u + 1;
                bool pass = true;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    int32_t d = cu[e] * mu + cw[e] * mw;
                    pass = pass && d >= lo[e] && d <= hi[e];
                }
                if (pass) mk |= 1ull << (u + 8 * w);
            }
        }
        mks[P] = mk;
    }
}

// A share of one (triangle, brick) item's setup: the cells of rows w = l0 + part, l0 + part + per, .. of the
// three projections' masks (OR-combined across the item's threads by the caller), and with do_plane the plane
// test and the item's fields.  Each item is spread over kItemLanes threads, so a large item's cell loops (up to
// 8 x 8 cells per projection) are not one thread's.
__device__ void item_part(const TriRec& r, const int64_t base[3], const int32_t l0[3], const int32_t l1[3], int part,
                          int per, bool do_plane, unsigned long long (&mks)[3], ItemSetup& out) {
    // brick-relative vertices and edges fit 32 bits (|q| < 2^19, base <= 2^17): products widen 32 x 32 -> 64
    int32_t v[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) v[a][b] = r.q[a * 3 + b] - int32_t(base[b]);
    // Items whose brick-relative vertices are below 2^14 in magnitude (a triangle within 64 voxels of the brick:
    // all but the largest) take the edge tests in 32-bit integers: edge components < 2^15, each product < 2^29, a
    // dot product (two nonzero terms) < 2^30, the box radius < 2^23, so nothing overflows and the bounds are the
    // same integers the 64-bit form computes.
    int32_t vmax = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) vmax = max(vmax, abs(v[a][b]));
    if (vmax < (1 << 14))
        item_masks<int32_t>(v, l0, l1, part, per, mks);
    else
        item_masks<int64_t>(v, l0, l1, part, per, mks);
    if (!do_plane) return;
    int32_t e0[3], e1[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) e0[b] = v[1][b] - v[0][b], e1[b] = v[2][b] - v[0][b];
    const int64_t n0 = int64_t(e0[1]) * e1[2] - int64_t(e0[2]) * e1[1], n1 = int64_t(e0[2]) * e1[0] - int64_t(e0[0]) * e1[2],
                  n2 = int64_t(e0[0]) * e1[1] - int64_t(e0[1]) * e1[0];
    const int64_t sp = n0 * v[0][0] + n1 * v[0][1] + n2 * v[0][2];
    const int64_t rr = kHalf * (iabs64(n0) + iabs64(n1) + iabs64(n2));
    out.n[0] = n0, out.n[1] = n1, out.n[2] = n2;
    out.plo = sar7_ceil(sp - rr);  // overlap iff sp - rr <= 128 (n . m) <= sp + rr
    out.phi = sar7_floor(sp + rr);
    const int64_t lim = int64_t(1) << 25;
    out.small = (iabs64(n0) < lim && iabs64(n1) < lim && iabs64(n2) < lim) ? 1 : 0;
    out.wq[0] = r.wq[0], out.wq[1] = r.wq[1], out.wq[2] = r.wq[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) out.l0[a] = uint8_t(l0[a]), out.ext[a] = uint8_t(l1[a] - l0[a] + 1);
}

// Adjacent lanes preparing one item in vox_items (per 500k-triangle voxelization: 4 lanes 0.615 ms, 2 lanes
// 0.590, 1 lane 0.588 with the bricks' CTAs otherwise the same: the shared rows save less than the repeated
// set-up of every lane costs)
constexpr int kItemLanes = 1;

// Every (triangle, brick) item of the lists, prepared apart from its brick: the three projections' cell masks
// (each of an item's kItemLanes lanes a share of the rows, OR-combined by shuffles), the plane test and the
// item's voxel box, written in list order for vox_bricks.  It needs the triangle records and the lists only, so it
// runs on the lists' stream beside the shadow raster, at full occupancy and with no barrier: prepared inside the
// brick's CTA, a large item's cell loops held the CTA's other threads at the barrier after them.
// Five CTAs of 256 threads per SM (48 registers): the items' loads wait on the list, then the triangle record, so
// the kernel wants warps more than registers (per 500k-triangle voxelization 0.598 ms at 80 registers, 3 CTAs
// per SM; 0.593 at 64, 4 per SM; 0.590 at 48).
__global__ void __launch_bounds__(256, 5) vox_items(uint32_t dim, uint64_t ntris, VoxScratch sc) {
    const uint32_t n = uint32_t(min(uint64_t(*sc.total), sc.list_cap));
    const uint32_t lane = threadIdx.x & 31, part = lane % kItemLanes;
    constexpr uint32_t kPerWarp = 32 / kItemLanes;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i0 = gw * kPerWarp; i0 < n; i0 += nw * kPerWarp) {  // warp-uniform rounds (full-mask shuffles)
        const uint32_t i = i0 + lane / kItemLanes;
        unsigned long long mks[3] = {0ull, 0ull, 0ull};
        ItemSetup it = {};  // an item whose voxel box misses its brick keeps ext = 0: no rows
        const uint32_t t = i < n ? sc.list[i] : 0u;
        if (i < n && t < ntris) {
            const uint32_t m = sc.list_brick[i];
            const TriRec r = sc.recs[t];
            const int32_t bx = int32_t(compact1by2(m)), by = int32_t(compact1by2(m >> 1)),
                          bz = int32_t(compact1by2(m >> 2));
            const int64_t base[3] = {int64_t(bx) * kBrickFix, int64_t(by) * kBrickFix, int64_t(bz) * kBrickFix};
            int32_t lo[3], hi[3];
            voxel_range(r.q, dim, lo, hi);
            const int32_t l0[3] = {max(lo[0], bx * 8) - bx * 8, max(lo[1], by * 8) - by * 8, max(lo[2], bz * 8) - bz * 8};
            const int32_t l1[3] = {min(hi[0], bx * 8 + 7) - bx * 8, min(hi[1], by * 8 + 7) - by * 8,
                                   min(hi[2], bz * 8 + 7) - bz * 8};
            if (l0[0] <= l1[0] && l0[1] <= l1[1] && l0[2] <= l1[2])
                item_part(r, base, l0, l1, int(part), kItemLanes, part == kItemLanes - 1, mks, it);
        }
#pragma unroll
        for (int P = 0; P < 3; ++P) {
            uint32_t mlo = uint32_t(mks[P]), mhi = uint32_t(mks[P] >> 32);
#pragma unroll
            for (int o = 1; o < kItemLanes; o <<= 1) {
                mlo |= __shfl_xor_sync(0xffffffffu, mlo, o);
                mhi |= __shfl_xor_sync(0xffffffffu, mhi, o);
            }
            it.mask[P] = (uint64_t(mhi) << 32) | mlo;
        }
        if (i < n && part == kItemLanes - 1) sc.items[i] = it;
    }
}

constexpr int kChunk = 128;  // items staged per round (one per thread; = threads per CTA)
constexpr uint32_t kRowCap = 1024;  // rows per round mapped to their item by table (later ones by search)

// Fourteen CTAs per SM (32 registers, 16 KB of shared memory each: the prepared items are read from global memory
// where a row needs them, not staged): a brick's phases are separated by barriers at which most of its threads
// wait, so other bricks' CTAs are what keeps the SM busy (per 500k-triangle voxelization: 0.59 -> 0.40 ms at 8
// CTAs per SM against 4, with the items prepared in the CTA; with the items prepared by vox_items, 8 CTAs staging
// them 0.588 ms, 10 / 12 / 14 CTAs reading them from global memory 0.578 / 0.572 / 0.565 ms).
__global__ void __launch_bounds__(kChunk, 14) vox_bricks(VoxScratch sc, const f184gi_grid_frame* __restrict__ fr,
                                                  uint32_t dim, ChainLayout chain, f184gi_light light,
                                                  const unsigned long long* __restrict__ shadow, uint32_t res,
                                                  uint32_t* counts, const uint32_t* __restrict__ dirty,
                                                  float4* __restrict__ weights, uint32_t nlow, uint32_t* status) {
    // Per voxel, 33.31 fixed-point sums of the three channels, exact and order-independent, as 32-bit words: the
    // low words (0..2) by atomic add, the high words (3..5) counting the low words' carries (shared-memory 32-bit
    // atomics run ~2.5x the rate of 64-bit ones).  With nlow > 0 a voxel's six words then hold its FP32 output
    // (two float2), which the brick's levels 1..nlow are reduced from.
    __shared__ __align__(16) uint32_t s_acc[512][6];
    __shared__ __align__(16) uint32_t s_cnt[512];  // then levels 1 and 2 of the brick (64 + 8 float4)
    __shared__ uint32_t s_start[kChunk + 1];       // prefix of x-rows per prepared item
    __shared__ uint8_t s_rowitem[kRowCap];         // item slot of each of the first kRowCap rows
    const uint32_t m = dirty ? dirty[blockIdx.x] : blockIdx.x;
    const uint32_t nb = dim >> 3;
    if (m >= nb * nb * nb) return;
    const int32_t bx = int32_t(compact1by2(m)), by = int32_t(compact1by2(m >> 1)), bz = int32_t(compact1by2(m >> 2));
    const uint32_t beg = sc.brick_start[m];
    const uint32_t end = uint32_t(min(uint64_t(beg) + sc.brick_count[m], sc.list_cap));
    if (beg == end) {  // an empty brick: zeros, without the shared-memory sums
        for (uint32_t j = threadIdx.x; j < 64u + 8u + 1u; j += kChunk) {  // its blocks of levels 1..nlow
            const uint32_t k = j < 64u ? 1u : (j < 72u ? 2u : 3u), e = j < 64u ? 1u << (3 - k) : j < 72u ? 2u : 1u;
            const uint32_t r = j - (k == 1u ? 0u : k == 2u ? 64u : 72u);
            if (k <= nlow)
                store_vox(chain.base, F184GI_FMT_F32,
                          chain.off[k] + vox_index(k, chain.ldim[k], uint32_t(bx) * e + r % e,
                                                   uint32_t(by) * e + (r / e) % e, uint32_t(bz) * e + r / (e * e)),
                          make_float4(0.f, 0.f, 0.f, 0.f));
        }
        for (int li = threadIdx.x; li < 512; li += kChunk) {
            if (weights)
                weights[(uint64_t(m) << 9) + li] = make_float4(0.f, 0.f, 0.f, 0.f);
            else
                store_vox(chain.base, chain.format, chain.off[0] + (uint64_t(m) << 9) + li, make_float4(0.f, 0.f, 0.f, 0.f));
            if (counts) {
                const int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
                counts[(uint64_t(bz * 8 + lz) * dim + uint64_t(by * 8 + ly)) * dim + uint64_t(bx * 8 + lx)] = 0;
            }
        }
        return;
    }
    for (int i = threadIdx.x; i < 512; i += kChunk) {
#pragma unroll
        for (int w = 0; w < 6; ++w) s_acc[i][w] = 0u;
        s_cnt[i] = 0;
    }
    for (uint32_t c0 = beg; c0 < end; c0 += kChunk) {
        // phase 1: the x-row counts of the chunk's prepared items (vox_items), one item per thread
        const uint32_t nchunk = min(end - c0, uint32_t(kChunk));
        uint32_t nrows = 0;
        if (threadIdx.x < nchunk) {
            const ItemSetup& it = sc.items[c0 + threadIdx.x];
            nrows = uint32_t(it.ext[1]) * uint32_t(it.ext[2]);
        }
        // exclusive scan of the row counts (warp shuffles + one pass over the 4 warp totals)
        {
            const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            uint32_t x = nrows;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= uint32_t(o)) x += y;
            }
            __shared__ uint32_t s_wsum[kChunk / 32];
            if (lane == 31) s_wsum[wid] = x;
            __syncthreads();
            uint32_t pre = 0;
            for (uint32_t w = 0; w < wid; ++w) pre += s_wsum[w];
            s_start[threadIdx.x] = pre + x - nrows;
            if (threadIdx.x == kChunk - 1) s_start[kChunk] = pre + x;
            __syncthreads();
        }
        const uint32_t total = s_start[kChunk];
        // the item of each of the first kRowCap rows, written by the item's thread (its rows are contiguous)
        if (nrows) {
            const uint32_t st = s_start[threadIdx.x];
            for (uint32_t j = 0; j < nrows && st + j < kRowCap; ++j) s_rowitem[st + j] = uint8_t(threadIdx.x);
        }
        __syncthreads();
        // phase 2: all threads share the x-rows (item, y, z) of the chunk's voxel boxes evenly.  A row's candidate
        // voxels are the bits of one byte: projection 2 holds x + 8y (byte y), projection 1 holds z + 8x (the
        // bits z, z + 8, .., z + 56, gathered into a byte by one multiply), projection 0 one bit y + 8z.
        for (uint32_t rr = threadIdx.x; rr < total; rr += blockDim.x) {
            uint32_t lo;  // the row's item: the k with s_start[k] <= rr < s_start[k + 1]
            if (rr < kRowCap) {
                lo = uint32_t(s_rowitem[rr]);
            } else {
                lo = 0;
                uint32_t hi = kChunk;
                while (hi - lo > 1) {
                    uint32_t mid = (lo + hi) >> 1;
                    if (s_start[mid] <= rr) lo = mid; else hi = mid;
                }
            }
            const ItemSetup& is = sc.items[c0 + lo];
            const uint32_t local = rr - s_start[lo];
            const uint32_t ey = is.ext[1];
            // local / ey for local < 64, ey <= 8: the quotient's fraction stays >= 1/16 from an integer
            const uint32_t qz = uint32_t((float(local) + 0.5f) * __frcp_rn(float(ey)));
            const int ly = is.l0[1] + int(local - qz * ey), lz = is.l0[2] + int(qz);
            if (!((is.mask[0] >> (ly + 8 * lz)) & 1ull)) continue;
            const uint32_t col = uint32_t((((is.mask[1] >> lz) & 0x0101010101010101ull) * 0x0102040810204080ull) >> 56);
            uint32_t xm = uint32_t(is.mask[2] >> (8 * ly)) & col & 0xffu;
            if (!xm) continue;
            // the plane test n . m within [plo, phi] for the row's candidates; with |n| < 2^25 each term is below
            // 15 * 2^25 and n . m below 2^31, so it runs in 32 bits against the bounds clamped to 32 bits (a bound
            // beyond the 32-bit range decides nothing for a 32-bit value): the same decisions
            uint32_t pass = 0;
            if (is.small) {
                const int32_t n0 = int32_t(is.n[0]);
                const int32_t drow = int32_t(is.n[1]) * (2 * ly + 1) + int32_t(is.n[2]) * (2 * lz + 1);
                const int32_t lo = int32_t(max(is.plo, (long long)INT32_MIN)), hi = int32_t(min(is.phi, (long long)INT32_MAX));
                for (uint32_t m = xm; m; m &= m - 1) {
                    const int lx = __ffs(m) - 1;
                    const int32_t d = n0 * (2 * lx + 1) + drow;
                    if (d >= lo && d <= hi) pass |= 1u << lx;
                }
            } else {
                const long long drow = is.n[1] * (2 * ly + 1) + is.n[2] * (2 * lz + 1);
                for (uint32_t m = xm; m; m &= m - 1) {
                    const int lx = __ffs(m) - 1;
                    const long long d = is.n[0] * (2 * lx + 1) + drow;
                    if (d >= is.plo && d <= is.phi) pass |= 1u << lx;
                }
            }
            while (pass) {
                const int lx = __ffs(pass) - 1;
                pass &= pass - 1;
                const int li = lz * 64 + ly * 8 + lx;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint32_t old = atomicAdd(&s_acc[li][c], is.wq[c]);
                    if (old + is.wq[c] < old) atomicAdd(&s_acc[li][3 + c], 1u);
                }
                atomicAdd(&s_cnt[li], 1u);
            }
        }
        __syncthreads();  // the next chunk rewrites the item table
    }
    __syncthreads();
    // resolve: radiance = luminance * shadow * mean weight, opacity 1 where covered
    for (int li = threadIdx.x; li < 512; li += kChunk) {
        int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
        uint32_t cnt = s_cnt[li];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (cnt) {
            // mean injection weight (FP32), then radiance = luminance * (lit ? weight : 0)
            const float q = (1.0f / 2147483648.0f) / float(cnt);
            const float4 w = make_float4(float((uint64_t(s_acc[li][3]) << 32) | s_acc[li][0]) * q,
                                         float((uint64_t(s_acc[li][4]) << 32) | s_acc[li][1]) * q,
                                         float((uint64_t(s_acc[li][5]) << 32) | s_acc[li][2]) * q, 1.0f);
            if (weights) {
                out = w;  // geometry only: relight_bricks applies the shadow test and the luminance
            } else {
                const bool lit = voxel_lit(fr, shadow, res, bx * 8 + lx, by * 8 + ly, bz * 8 + lz);
                out = make_float4(light.luminance[0] * (lit ? w.x : 0.0f), light.luminance[1] * (lit ? w.y : 0.0f),
                                  light.luminance[2] * (lit ? w.z : 0.0f), 1.0f);
            }
        }
        if (weights)
            weights[(uint64_t(m) << 9) + li] = out;
        else
            store_vox(chain.base, chain.format, chain.off[0] + (uint64_t(m) << 9) + li, out);
        if (counts) {
            uint64_t lin = (uint64_t(bz * 8 + lz) * dim + uint64_t(by * 8 + ly)) * dim + uint64_t(bx * 8 + lx);
            counts[lin] = cnt;
        }
        if (nlow) {  // the output over the voxel's own sums (read above by this thread only)
            float2* slot = reinterpret_cast<float2*>(s_acc[li]);
            slot[0] = make_float2(out.x, out.y);
            slot[1] = make_float2(out.z, out.w);
        }
    }
    if (!nlow) return;
    // The brick's blocks of levels 1..nlow (4^3, 2^3, 1), each voxel the mean of its 2x2x2 children (iso_mean8,
    // as the mip kernels compute them, hence the same bytes): level 1 from the brick's FP32 outputs, level 2 from
    // level 1's FP32 values, level 3 from level 2's.
    float4* s_l1 = reinterpret_cast<float4*>(s_cnt);
    float4* s_l2 = s_l1 + 64;
    __syncthreads();
    if (threadIdx.x < 64) {
        const uint32_t x = threadIdx.x & 3u, y = (threadIdx.x >> 2) & 3u, z = threadIdx.x >> 4;
        const float4 v = iso_mean8([&](int dx, int dy, int dz) {
            const float2* c = reinterpret_cast<const float2*>(s_acc[((2 * z + dz) << 6) + ((2 * y + dy) << 3) + 2 * x + dx]);
            const float2 a = c[0], b = c[1];
            return make_float4(a.x, a.y, b.x, b.y);
        });
        s_l1[threadIdx.x] = v;
        store_vox(chain.base, F184GI_FMT_F32,
                  chain.off[1] + vox_index(1, chain.ldim[1], uint32_t(bx) * 4 + x, uint32_t(by) * 4 + y, uint32_t(bz) * 4 + z), v);
    }
    if (nlow < 2) return;
    __syncthreads();
    if (threadIdx.x < 8) {
        const uint32_t x = threadIdx.x & 1u, y = (threadIdx.x >> 1) & 1u, z = threadIdx.x >> 2;
        const float4 v = iso_mean8([&](int dx, int dy, int dz) { return s_l1[((2 * z + dz) << 4) + ((2 * y + dy) << 2) + 2 * x + dx]; });
        s_l2[threadIdx.x] = v;
        store_vox(chain.base, F184GI_FMT_F32,
                  chain.off[2] + vox_index(2, chain.ldim[2], uint32_t(bx) * 2 + x, uint32_t(by) * 2 + y, uint32_t(bz) * 2 + z), v);
    }
    if (nlow < 3) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        const float4 v = iso_mean8([&](int dx, int dy, int dz) { return s_l2[(dz << 2) + (dy << 1) + dx]; });
        store_vox(chain.base, F184GI_FMT_F32, chain.off[3] + vox_index(3, chain.ldim[3], uint32_t(bx), uint32_t(by), uint32_t(bz)), v);
    }
}

template <class T>
T* carve(char*& p, uint64_t n) {
    uintptr_t a = (reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255);
    T* r = reinterpret_cast<T*>(a);
    p = reinterpret_cast<char*>(a + n * sizeof(T));
    return r;
}

uint64_t list_capacity(uint64_t ntris, uint32_t nbricks) { return ntris * 6 + uint64_t(nbricks) * 2 + 65536; }

bool g_lut_ready = false;

}  // namespace

size_t voxelize_scratch_bytes(uint64_t ntris, uint32_t dim) {
    uint32_t nb = dim / 8, nbricks = nb * nb * nb;
    return ntris * sizeof(TriRec) + uint64_t(nbricks) * 12 + scan_scratch_bytes(nbricks) + (nbricks / 32 + 1) * 4 +
           list_capacity(ntris, nbricks) * (8 + sizeof(ItemSetup)) + (ntris + 2) * 4 + (ntris + 2) * 4 + (ntris + 1) * 8 + ntris + 24 * 256;
}

namespace {

// The scratch layout shared by the two phases.
VoxScratch carve_scratch(const VoxelizeJob& job, void* scratch, uint32_t** mask) {
    const uint32_t nb = job.chain.dim / 8, nbricks = nb * nb * nb;
    char* p = static_cast<char*>(scratch);
    VoxScratch sc;
    sc.recs = carve<TriRec>(p, job.ntris);
    sc.brick_count = carve<uint32_t>(p, nbricks);
    sc.brick_start = carve<uint32_t>(p, nbricks);
    sc.brick_fill = carve<uint32_t>(p, nbricks);
    sc.total = carve<uint32_t>(p, 1);
    sc.scan_tmp = carve<uint32_t>(p, scan_scratch_bytes(nbricks) / 4);
    *mask = carve<uint32_t>(p, nbricks / 32 + 1);
    sc.list_cap = list_capacity(job.ntris, nbricks);
    sc.list = carve<uint32_t>(p, sc.list_cap);
    sc.list_brick = carve<uint32_t>(p, sc.list_cap);
    sc.items = carve<ItemSetup>(p, sc.list_cap);
    sc.big = carve<uint32_t>(p, job.ntris + 1);
    sc.big_count = carve<uint32_t>(p, 1);
    sc.mid = carve<uint32_t>(p, job.ntris + 1);
    sc.mid_count = carve<uint32_t>(p, 1);
    sc.mid_bits = carve<uint2>(p, job.ntris + 1);
    sc.bits = carve<uint8_t>(p, job.ntris);
    sc.dirty_mask = job.ndirty ? *mask : nullptr;
    return sc;
}

int check_job(const VoxelizeJob& job, size_t scratch_bytes) {
    const uint32_t dim = job.chain.dim;
    if (dim < 16 || dim > 512 || (dim & (dim - 1))) return fail(F184GI_ERR_INVALID, "voxelize: dim must be 2^k in 16..512");
    if (job.ntris >= 0xffff0000ull) return fail(F184GI_ERR_INVALID, "voxelize: too many triangles");
    if (scratch_bytes < voxelize_scratch_bytes(job.ntris, dim)) return fail(F184GI_ERR_INVALID, "voxelize: scratch too small");
    return F184GI_OK;
}

}  // namespace

int voxelize_lists_launch(const VoxelizeJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                          cudaStream_t s) {
    int rc = check_job(job, scratch_bytes);
    if (rc) return rc;
    const uint32_t dim = job.chain.dim;
    if (!g_lut_ready) {
        float lut[256];
        for (int i = 0; i < 256; ++i) lut[i] = float(std::pow(double(i) / 255.0, 2.2));
        cudaError_t e = cudaMemcpyToSymbol(c_albedo_lut, lut, sizeof(lut));
        if (e != cudaSuccess) return cuda_fail(e, "voxelize: albedo table");
        g_lut_ready = true;
    }
    const uint32_t nb = dim / 8, nbricks = nb * nb * nb;
    uint32_t* mask = nullptr;
    VoxScratch sc = carve_scratch(job, scratch, &mask);
    cudaMemsetAsync(sc.big_count, 0, 4, s);
    cudaMemsetAsync(sc.mid_count, 0, 4, s);
    cudaMemsetAsync(sc.brick_count, 0, size_t(nbricks) * 4, s);
    cudaMemsetAsync(sc.brick_fill, 0, size_t(nbricks) * 4, s);
    if (job.ndirty) {
        cudaMemsetAsync(mask, 0, size_t(nbricks / 32 + 1) * 4, s);
        vox_dirty_mask<<<(job.ndirty + 255) / 256, 256, 0, s>>>(job.dirty_bricks, job.ndirty, nbricks, mask);
        note_launches(1);
    }
    if (job.ntris) {
        vox_setup<<<uint32_t((job.ntris + 127) / 128), 128, 0, s>>>(job.tri, job.albedo, job.ntris, job.d_frame, dim,
                                                                     sc, d_status);
        vox_bin_big<<<8 * 152, 256, 0, s>>>(dim, sc, d_status, 0);
        note_launches(2);
    }
    if ((rc = exclusive_scan(sc.brick_count, nbricks, sc.brick_start, sc.total, sc.scan_tmp, s))) return rc;
    if (job.ntris) {
        vox_emit<<<uint32_t((job.ntris + 127) / 128), 128, 0, s>>>(job.ntris, dim, sc, d_status);
        vox_bin_big<<<8 * 152, 256, 0, s>>>(dim, sc, d_status, 1);
        vox_items<<<8 * 152, 256, 0, s>>>(dim, job.ntris, sc);
        note_launches(3);
    }
    return cuda_fail(cudaGetLastError(), "voxelize lists");
}

int voxelize_bricks_launch(const VoxelizeJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                           cudaStream_t s) {
    int rc = check_job(job, scratch_bytes);
    if (rc) return rc;
    const uint32_t dim = job.chain.dim, nb = dim / 8, nbricks = nb * nb * nb;
    uint32_t* mask = nullptr;
    VoxScratch sc = carve_scratch(job, scratch, &mask);
    const uint32_t nblocks = job.ndirty ? job.ndirty : nbricks;
    vox_bricks<<<nblocks, kChunk, 0, s>>>(sc, job.d_frame, dim, job.chain, job.light, job.shadow_keys, job.shadow_res,
                                       job.counts, job.ndirty ? job.dirty_bricks : nullptr, job.weights,
                                       job.weights ? 0u : job.mip_levels, d_status);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "voxelize");
}


}  // namespace f184

namespace f184 {
int relight_launch(const float4* weights, const f184gi_grid_frame* d_frame, const ChainLayout& chain,
                   const f184gi_light& light, const unsigned long long* shadow, uint32_t res, cudaStream_t s) {
    relight_bricks<<<152 * 8, 256, 0, s>>>(weights, d_frame, chain.dim, chain, light, shadow, res);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "relight");
}
}  // namespace f184
