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
// Pipeline: setup (snap, weight, count overlapped bricks) -> scan -> emit (triangle lists per brick) ->
// one CTA per brick accumulates in shared memory, resolves and writes the brick once.
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

struct TriRec {
    int32_t q[9];    // snapped vertices (x0 y0 z0 x1 ...), 24.8 voxel fixed point
    uint32_t wq[3];  // injection weight per channel, 1.31 fixed point (<= 2^31); wq[0] = kInvalid marks skipped
};

struct VoxScratch {
    TriRec* recs;
    uint32_t* brick_count;
    uint32_t* brick_start;
    uint32_t* brick_fill;
    uint32_t* total;
    uint32_t* scan_tmp;
    uint32_t* dirty_mask;  // nbricks bits, null = all bricks
    uint32_t* list;
    uint32_t* big;        // triangles with more than kWarpCells bricks (binned by vox_bin_big)
    uint32_t* big_count;  // [1]
    uint64_t list_cap;
};

__device__ __forceinline__ int64_t iabs64(int64_t x) { return x < 0 ? -x : x; }
__device__ __forceinline__ int64_t sar7_floor(int64_t x) { return x >> 7; }         // floor(x / 128)
__device__ __forceinline__ int64_t sar7_ceil(int64_t x) { return -((-x) >> 7); }    // ceil(x / 128)
__device__ __forceinline__ int32_t clamp32(int64_t x) {
    return int32_t(x > int64_t(INT32_MAX) ? int64_t(INT32_MAX) : (x < int64_t(INT32_MIN) ? int64_t(INT32_MIN) : x));
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
    for (int e = 0; e < 3; ++e) {
        int64_t ed[3];
        for (int b = 0; b < 3; ++b) ed[b] = v[(e + 1) % 3][b] - v[e][b];
        for (int ax = 0; ax < 3; ++ax) {
            int64_t a0 = 0, a1 = 0, a2 = 0;
            if (ax == 0) a1 = ed[2], a2 = -ed[1];
            if (ax == 1) a0 = -ed[2], a2 = ed[0];
            if (ax == 2) a0 = ed[1], a1 = -ed[0];
            int64_t p0 = a0 * v[0][0] + a1 * v[0][1] + a2 * v[0][2];
            int64_t p1 = a0 * v[1][0] + a1 * v[1][1] + a2 * v[1][2];
            int64_t p2 = a0 * v[2][0] + a1 * v[2][1] + a2 * v[2][2];
            int64_t rr = h * (iabs64(a0) + iabs64(a1) + iabs64(a2));
            if (min(p0, min(p1, p2)) > rr || max(p0, max(p1, p2)) < -rr) return false;
        }
    }
    return true;
}

// voxel range touched by the triangle's AABB (closed boxes), clamped to the grid
__device__ __forceinline__ void voxel_range(const int32_t* q, uint32_t dim, int32_t lo[3], int32_t hi[3]) {
    for (int a = 0; a < 3; ++a) {
        int64_t mn = min(q[a], min(q[3 + a], q[6 + a])), mx = max(q[a], max(q[3 + a], q[6 + a]));
        lo[a] = int32_t(max(int64_t(0), -floor_div64(-(mn - kFix), kFix)));
        hi[a] = int32_t(min(int64_t(dim) - 1, floor_div64(mx, kFix)));
    }
}

constexpr int kWarpCells = 8;  // triangles overlapping more bricks than this are binned by a whole CTA

__device__ __forceinline__ void bin_brick(const int32_t* q, uint32_t t, int bx, int by, int bz, bool test,
                                          const VoxScratch& sc, uint32_t* status, bool emit) {
    uint32_t m = morton3(bx, by, bz);
    if (sc.dirty_mask && !((sc.dirty_mask[m >> 5] >> (m & 31)) & 1u)) return;
    if (test) {
        const int64_t c[3] = {bx * kBrickFix + kBrickFix / 2, by * kBrickFix + kBrickFix / 2,
                              bz * kBrickFix + kBrickFix / 2};
        if (!tri_box_sat(q, c, kBrickFix / 2)) return;
    }
    if (!emit) {
        atomicAdd(&sc.brick_count[m], 1u);
    } else {
        uint64_t slot = uint64_t(sc.brick_start[m]) + atomicAdd(&sc.brick_fill[m], 1u);
        if (slot < sc.list_cap)
            sc.list[slot] = t;
        else
            set_status(status, kStatusOverflow);
    }
}

// brick box of a triangle: first brick and extent per axis
__device__ __forceinline__ int brick_box(const int32_t* q, uint32_t dim, int32_t b0[3], int32_t nb[3]) {
    int32_t lo[3], hi[3];
    voxel_range(q, dim, lo, hi);
    for (int a = 0; a < 3; ++a) b0[a] = lo[a] >> 3, nb[a] = (hi[a] >> 3) - b0[a] + 1;
    return nb[0] * nb[1] * nb[2];
}

// Count (emit = false) or list (emit = true) the bricks of a triangle with at most kWarpCells bricks; larger
// triangles are queued on the count pass and binned by vox_bin_big (one CTA per triangle).
__device__ __forceinline__ void bin_small(const TriRec& r, uint32_t t, uint32_t dim, const VoxScratch& sc,
                                          uint32_t* status, bool emit, uint64_t ntris) {
    int32_t b0[3], nb[3];
    const int ncell = brick_box(r.q, dim, b0, nb);
    if (ncell > kWarpCells) {
        if (!emit) {
            uint32_t k = atomicAdd(sc.big_count, 1u);
            if (k < ntris) sc.big[k] = t;
        }
        return;
    }
    for (int c = 0; c < ncell; ++c)
        bin_brick(r.q, t, b0[0] + c % nb[0], b0[1] + (c / nb[0]) % nb[1], b0[2] + c / (nb[0] * nb[1]), ncell > 1, sc,
                  status, emit);
}

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
}

__global__ void __launch_bounds__(128) vox_setup(const float* __restrict__ tri, const uint32_t* __restrict__ albedo,
                                                 uint64_t ntris, const f184gi_grid_frame* __restrict__ fr, uint32_t dim,
                                                 VoxScratch sc, uint32_t* status) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    TriRec r;
    bool ok = t < ntris;
    const float* p = tri + (ok ? t : 0) * 9;
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
        float len = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
        float wi0 = -float(fr->light_dir[0]), wi1 = -float(fr->light_dir[1]), wi2 = -float(fr->light_dir[2]);
        float cosv = len > 0.0f ? fabsf(wi0 * n.x + wi1 * n.y + wi2 * n.z) / len : 0.0f;
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

constexpr int kSmallVox = 64;       // items with at most this many candidate voxels run on one thread
constexpr uint32_t kLargeCap = 512;  // per-brick queue of warp-shared items (overflow runs on one thread)

// One thread tests every candidate voxel of a (triangle, brick) item; l0..l1 is the item's voxel box in brick
// coordinates.  The same exact tests as the warp path: edge axes crossed with x depend only on (y, z), so they
// are hoisted out of the x loop.
__device__ __forceinline__ void item_thread(const TriRec& r, const int64_t base[3], const int32_t l0[3],
                                            const int32_t l1[3], unsigned long long (*s_sum)[512], uint32_t* s_cnt) {
    int64_t v[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) v[a][b] = int64_t(r.q[a * 3 + b]) - base[b];
    // nine edge axes: a = edge x unit(ax); keep its two non-zero components (|a| < 2^21) and the bounds
    int32_t c1[9], c2[9], alo[9], ahi[9];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        int64_t ed[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) ed[b] = v[(e + 1) % 3][b] - v[e][b];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            int64_t a0 = 0, a1 = 0, a2 = 0;
            if (ax == 0) a1 = ed[2], a2 = -ed[1];
            if (ax == 1) a0 = -ed[2], a2 = ed[0];
            if (ax == 2) a0 = ed[1], a1 = -ed[0];
            int64_t p0 = a0 * v[0][0] + a1 * v[0][1] + a2 * v[0][2];
            int64_t p1 = a0 * v[1][0] + a1 * v[1][1] + a2 * v[1][2];
            int64_t p2 = a0 * v[2][0] + a1 * v[2][1] + a2 * v[2][2];
            int64_t rr = kHalf * (iabs64(a0) + iabs64(a1) + iabs64(a2));
            int64_t pmin = min(p0, min(p1, p2)), pmax = max(p0, max(p1, p2));
            const int k = e * 3 + ax;
            // ax 0: (y, z) components; ax 1: (x, z); ax 2: (x, y)
            c1[k] = int32_t(ax == 0 ? a1 : a0);
            c2[k] = int32_t(ax == 2 ? a1 : a2);
            alo[k] = clamp32(sar7_ceil(pmin - rr));
            ahi[k] = clamp32(sar7_floor(pmax + rr));
        }
    }
    int64_t e0[3], e1[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) e0[b] = v[1][b] - v[0][b], e1[b] = v[2][b] - v[0][b];
    const int64_t n0 = e0[1] * e1[2] - e0[2] * e1[1], n1 = e0[2] * e1[0] - e0[0] * e1[2],
                  n2 = e0[0] * e1[1] - e0[1] * e1[0];
    const int64_t s = n0 * v[0][0] + n1 * v[0][1] + n2 * v[0][2];
    const int64_t rr = kHalf * (iabs64(n0) + iabs64(n1) + iabs64(n2));
    const int64_t plo = sar7_ceil(s - rr), phi = sar7_floor(s + rr);
    const uint32_t w0 = r.wq[0], w1 = r.wq[1], w2 = r.wq[2];
    for (int lz = l0[2]; lz <= l1[2]; ++lz) {
        const int32_t mz = 2 * lz + 1;
        for (int ly = l0[1]; ly <= l1[1]; ++ly) {
            const int32_t my = 2 * ly + 1;
            bool row = true;
#pragma unroll
            for (int e = 0; e < 3; ++e) {  // x-crossed axes: independent of x
                const int k = e * 3;
                int32_t d = c1[k] * my + c2[k] * mz;
                row = row && d >= alo[k] && d <= ahi[k];
            }
            if (!row) continue;
            const int64_t pyz = n1 * my + n2 * mz;
            for (int lx = l0[0]; lx <= l1[0]; ++lx) {
                const int32_t mx = 2 * lx + 1;
                bool hit = true;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const int k1 = e * 3 + 1, k2 = e * 3 + 2;
                    int32_t d1 = c1[k1] * mx + c2[k1] * mz;  // (x, z)
                    int32_t d2 = c1[k2] * mx + c2[k2] * my;  // (x, y)
                    hit = hit && d1 >= alo[k1] && d1 <= ahi[k1] && d2 >= alo[k2] && d2 <= ahi[k2];
                }
                if (!hit) continue;
                const int64_t pd = pyz + n0 * mx;
                if (pd < plo || pd > phi) continue;
                const int li = lz * 64 + ly * 8 + lx;
                atomicAdd(&s_sum[0][li], (unsigned long long)w0);
                atomicAdd(&s_sum[1][li], (unsigned long long)w1);
                atomicAdd(&s_sum[2][li], (unsigned long long)w2);
                atomicAdd(&s_cnt[li], 1u);
            }
        }
    }
}

// Separating-axis tests of one (triangle, brick) item.  With m = 2 (voxel - brick origin) + 1 (odd, 1..15) the
// voxel centre is 128 m + brick offset, and each test reads lo <= a . m <= hi (exact integers).  The nine
// edge x unit-axis tests each ignore one coordinate, so they are evaluated once per cell of three 8x8
// projections into bit masks; a voxel is covered when its three projection bits and the plane test pass.

__global__ void __launch_bounds__(256, 2) vox_bricks(VoxScratch sc, const f184gi_grid_frame* __restrict__ fr,
                                                  uint32_t dim, ChainLayout chain, f184gi_light light,
                                                  const unsigned long long* __restrict__ shadow, uint32_t res,
                                                  uint32_t* counts, const uint32_t* __restrict__ dirty,
                                                  uint32_t* status) {
    __shared__ unsigned long long s_sum[3][512];  // 33.31 fixed point: exact, order-independent sums
    __shared__ uint32_t s_cnt[512];
    __shared__ int32_t s_ax[8][9][5];                // per warp: the nine edge-axis tests of its current item
    __shared__ unsigned long long s_mask[8][3];      // per warp: projection masks of its current item
    __shared__ uint32_t s_large[kLargeCap];          // list positions of items handled by whole warps
    __shared__ uint32_t s_nlarge;
    if (threadIdx.x == 0) s_nlarge = 0;
    const uint32_t m = dirty ? dirty[blockIdx.x] : blockIdx.x;
    const uint32_t nb = dim >> 3;
    if (m >= nb * nb * nb) return;
    const int32_t bx = int32_t(compact1by2(m)), by = int32_t(compact1by2(m >> 1)), bz = int32_t(compact1by2(m >> 2));
    for (int i = threadIdx.x; i < 512; i += 256) {
        s_sum[0][i] = s_sum[1][i] = s_sum[2][i] = 0;
        s_cnt[i] = 0;
    }
    __syncthreads();
    const uint32_t beg = sc.brick_start[m];
    const uint32_t end = uint32_t(min(uint64_t(beg) + sc.brick_count[m], sc.list_cap));
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base[3] = {int64_t(bx) * kBrickFix, int64_t(by) * kBrickFix, int64_t(bz) * kBrickFix};
    // Phase A: one thread per item whose box inside the brick has at most kSmallVox voxels (most items);
    // larger items are queued for Phase B, where a whole warp shares one item.
    for (uint32_t it = beg + threadIdx.x; it < end; it += blockDim.x) {
        const TriRec r = sc.recs[sc.list[it]];
        int32_t lo[3], hi[3];
        voxel_range(r.q, dim, lo, hi);
        lo[0] = max(lo[0], bx * 8), hi[0] = min(hi[0], bx * 8 + 7);
        lo[1] = max(lo[1], by * 8), hi[1] = min(hi[1], by * 8 + 7);
        lo[2] = max(lo[2], bz * 8), hi[2] = min(hi[2], bz * 8 + 7);
        if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) continue;
        const int vol = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
        if (vol > kSmallVox) {
            uint32_t k = atomicAdd(&s_nlarge, 1u);
            if (k < kLargeCap) {
                s_large[k] = it;
                continue;
            }
        }
        const int32_t l0[3] = {lo[0] - bx * 8, lo[1] - by * 8, lo[2] - bz * 8};
        const int32_t l1[3] = {hi[0] - bx * 8, hi[1] - by * 8, hi[2] - bz * 8};
        item_thread(r, base, l0, l1, s_sum, s_cnt);
    }
    __syncthreads();
    const uint32_t nlarge = min(s_nlarge, kLargeCap);
    // Phase B: warp-shared large items
    for (uint32_t k = warp; k < nlarge; k += 8) {
        const TriRec r = sc.recs[sc.list[s_large[k]]];
        int32_t lo[3], hi[3];
        voxel_range(r.q, dim, lo, hi);
        lo[0] = max(lo[0], bx * 8), hi[0] = min(hi[0], bx * 8 + 7);
        lo[1] = max(lo[1], by * 8), hi[1] = min(hi[1], by * 8 + 7);
        lo[2] = max(lo[2], bz * 8), hi[2] = min(hi[2], bz * 8 + 7);
        // vertices relative to the brick origin (|v| < 2^20)
        int64_t v[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) v[a][b] = int64_t(r.q[a * 3 + b]) - base[b];
        // lanes 0..8: edge e = lane / 3 crossed with unit axis P = lane % 3 (the projection it belongs to)
        if (lane < 9) {
            const int e = int(lane) / 3, ax = int(lane) % 3;
            int64_t ed[3];
#pragma unroll
            for (int b = 0; b < 3; ++b)  // edge e: v[e] -> v[(e + 1) % 3], selected without local-memory indexing
                ed[b] = e == 0 ? v[1][b] - v[0][b] : (e == 1 ? v[2][b] - v[1][b] : v[0][b] - v[2][b]);
            int64_t a0 = 0, a1 = 0, a2 = 0;
            if (ax == 0) a1 = ed[2], a2 = -ed[1];
            if (ax == 1) a0 = -ed[2], a2 = ed[0];
            if (ax == 2) a0 = ed[1], a1 = -ed[0];
            int64_t p0 = a0 * v[0][0] + a1 * v[0][1] + a2 * v[0][2];
            int64_t p1 = a0 * v[1][0] + a1 * v[1][1] + a2 * v[1][2];
            int64_t p2 = a0 * v[2][0] + a1 * v[2][1] + a2 * v[2][2];
            int64_t rr = kHalf * (iabs64(a0) + iabs64(a1) + iabs64(a2));
            int64_t pmin = min(p0, min(p1, p2)), pmax = max(p0, max(p1, p2));
            // overlap iff pmin - rr <= 128 (a . m) <= pmax + rr
            int32_t* sa = s_ax[warp][lane];
            sa[0] = int32_t(a0), sa[1] = int32_t(a1), sa[2] = int32_t(a2);
            sa[3] = clamp32(sar7_ceil(pmin - rr));
            sa[4] = clamp32(sar7_floor(pmax + rr));
        }
        if (lane < 3) s_mask[warp][lane] = 0ull;
        int64_t pn[3], plo, phi;
        {
            int64_t e0[3], e1[3];
            for (int b = 0; b < 3; ++b) {
                e0[b] = v[1][b] - v[0][b];
                e1[b] = v[2][b] - v[0][b];
            }
            pn[0] = e0[1] * e1[2] - e0[2] * e1[1];
            pn[1] = e0[2] * e1[0] - e0[0] * e1[2];
            pn[2] = e0[0] * e1[1] - e0[1] * e1[0];
            int64_t s = pn[0] * v[0][0] + pn[1] * v[0][1] + pn[2] * v[0][2];
            int64_t rr = kHalf * (iabs64(pn[0]) + iabs64(pn[1]) + iabs64(pn[2]));
            // overlap iff s - rr <= 128 (n . m) <= s + rr
            plo = sar7_ceil(s - rr);
            phi = sar7_floor(s + rr);
        }
        __syncwarp();
        const int l0x = lo[0] - bx * 8, l0y = lo[1] - by * 8, l0z = lo[2] - bz * 8;
        const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
        // projection cells: P = 0 -> (y, z), P = 1 -> (z, x), P = 2 -> (x, y)
        const int n0 = ny * nz, n1 = nz * nx, n2 = nx * ny;
        for (int e = int(lane); e < n0 + n1 + n2; e += 32) {
            int P, u, w;  // u, w: local coordinates of the two kept axes, bit = u + 8 w
            if (e < n0) {
                P = 0, u = l0y + e % ny, w = l0z + e / ny;
            } else if (e < n0 + n1) {
                int c = e - n0;
                P = 1, u = l0z + c % nz, w = l0x + c / nz;
            } else {
                int c = e - n0 - n1;
                P = 2, u = l0x + c % nx, w = l0y + c / nx;
            }
            // m along the two kept axes (the dropped axis has a zero coefficient in these tests)
            const int32_t mu = 2 * u + 1, mw = 2 * w + 1;
            const int32_t mx = P == 0 ? 0 : (P == 1 ? mw : mu);
            const int32_t my = P == 0 ? mu : (P == 1 ? 0 : mw);
            const int32_t mz = P == 0 ? mw : (P == 1 ? mu : 0);
            bool pass = true;
#pragma unroll
            for (int edge = 0; edge < 3; ++edge) {
                const int32_t* sa = s_ax[warp][edge * 3 + P];
                int32_t d = sa[0] * mx + sa[1] * my + sa[2] * mz;
                pass = pass && d >= sa[3] && d <= sa[4];
            }
            if (pass) atomicOr(&s_mask[warp][P], 1ull << (u + 8 * w));
        }
        __syncwarp();
        const unsigned long long mk0 = s_mask[warp][0], mk1 = s_mask[warp][1], mk2 = s_mask[warp][2];
        const int nvox = nx * ny * nz;
        for (int p = int(lane); p < nvox; p += 32) {
            int lx = l0x + p % nx, ly = l0y + (p / nx) % ny, lz = l0z + p / (nx * ny);
            bool hit = ((mk0 >> (ly + 8 * lz)) & (mk1 >> (lz + 8 * lx)) & (mk2 >> (lx + 8 * ly)) & 1ull) != 0;
            if (hit) {
                int64_t d = pn[0] * (2 * lx + 1) + pn[1] * (2 * ly + 1) + pn[2] * (2 * lz + 1);
                hit = d >= plo && d <= phi;
            }
            if (hit) {
                int li = lz * 64 + ly * 8 + lx;
                atomicAdd(&s_sum[0][li], (unsigned long long)r.wq[0]);
                atomicAdd(&s_sum[1][li], (unsigned long long)r.wq[1]);
                atomicAdd(&s_sum[2][li], (unsigned long long)r.wq[2]);
                atomicAdd(&s_cnt[li], 1u);
            }
        }
        __syncwarp();  // the next item rewrites this warp's axis table and masks
    }
    __syncthreads();
    // resolve: radiance = luminance * shadow * mean weight, opacity 1 where covered
    const float* lv = fr->light_vox;
    const float half_res = 0.5f * float(res);
    const float bias = fr->shadow_bias_f;
    for (int li = threadIdx.x; li < 512; li += 256) {
        int lx = li & 7, ly = (li >> 3) & 7, lz = li >> 6;
        uint32_t cnt = s_cnt[li];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        if (cnt) {
            // shadow test of the voxel centre: exact FP32 operation sequence (see frame.h)
            float fi = float(bx * 8 + lx), fj = float(by * 8 + ly), fk = float(bz * 8 + lz);
            float v[3];
#pragma unroll
            for (int rr = 0; rr < 3; ++rr) {
                const float* c = lv + 4 * rr;
                float s = __fadd_rn(c[0], __fmul_rn(fi, c[1]));
                s = __fadd_rn(s, __fmul_rn(fj, c[2]));
                v[rr] = __fadd_rn(s, __fmul_rn(fk, c[3]));
            }
            float tx = floorf(__fmul_rn(__fadd_rn(v[0], 1.0f), half_res));
            float ty = floorf(__fmul_rn(__fadd_rn(v[1], 1.0f), half_res));
            bool lit = true;
            if (tx >= 0.0f && ty >= 0.0f && tx < float(res) && ty < float(res)) {
                unsigned long long k = shadow[uint64_t(ty) * res + uint64_t(tx)];
                float sd = k == ~0ull ? 1.0f : __uint_as_float(uint32_t(k >> 32));
                lit = __fsub_rn(v[2], bias) <= sd;
            }
            float scale = lit ? (1.0f / 2147483648.0f) / float(cnt) : 0.0f;
            out.x = light.luminance[0] * (float(s_sum[0][li]) * scale);
            out.y = light.luminance[1] * (float(s_sum[1][li]) * scale);
            out.z = light.luminance[2] * (float(s_sum[2][li]) * scale);
            out.w = 1.0f;
        }
        store_vox(chain.base, chain.format, chain.off[0] + (uint64_t(m) << 9) + li, out);
        if (counts) {
            uint64_t lin = (uint64_t(bz * 8 + lz) * dim + uint64_t(by * 8 + ly)) * dim + uint64_t(bx * 8 + lx);
            counts[lin] = cnt;
        }
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
           list_capacity(ntris, nbricks) * 4 + (ntris + 2) * 4 + 20 * 256;
}

int voxelize_launch(const VoxelizeJob& job, void* scratch, size_t scratch_bytes, uint32_t* d_status, cudaStream_t s) {
    const uint32_t dim = job.chain.dim;
    if (dim < 16 || dim > 512 || (dim & (dim - 1))) return fail(F184GI_ERR_INVALID, "voxelize: dim must be 2^k in 16..512");
    if (job.ntris >= 0xffff0000ull) return fail(F184GI_ERR_INVALID, "voxelize: too many triangles");
    if (scratch_bytes < voxelize_scratch_bytes(job.ntris, dim)) return fail(F184GI_ERR_INVALID, "voxelize: scratch too small");
    if (!g_lut_ready) {
        float lut[256];
        for (int i = 0; i < 256; ++i) lut[i] = float(std::pow(double(i) / 255.0, 2.2));
        cudaError_t e = cudaMemcpyToSymbol(c_albedo_lut, lut, sizeof(lut));
        if (e != cudaSuccess) return cuda_fail(e, "voxelize: albedo table");
        g_lut_ready = true;
    }
    const uint32_t nb = dim / 8, nbricks = nb * nb * nb;
    char* p = static_cast<char*>(scratch);
    VoxScratch sc;
    sc.recs = carve<TriRec>(p, job.ntris);
    sc.brick_count = carve<uint32_t>(p, nbricks);
    sc.brick_start = carve<uint32_t>(p, nbricks);
    sc.brick_fill = carve<uint32_t>(p, nbricks);
    sc.total = carve<uint32_t>(p, 1);
    sc.scan_tmp = carve<uint32_t>(p, scan_scratch_bytes(nbricks) / 4);
    uint32_t* mask = carve<uint32_t>(p, nbricks / 32 + 1);
    sc.list_cap = list_capacity(job.ntris, nbricks);
    sc.list = carve<uint32_t>(p, sc.list_cap);
    sc.big = carve<uint32_t>(p, job.ntris + 1);
    sc.big_count = carve<uint32_t>(p, 1);
    sc.dirty_mask = nullptr;
    cudaMemsetAsync(sc.big_count, 0, 4, s);
    cudaMemsetAsync(sc.brick_count, 0, size_t(nbricks) * 4, s);
    cudaMemsetAsync(sc.brick_fill, 0, size_t(nbricks) * 4, s);
    if (job.ndirty) {
        sc.dirty_mask = mask;
        cudaMemsetAsync(mask, 0, size_t(nbricks / 32 + 1) * 4, s);
        vox_dirty_mask<<<(job.ndirty + 255) / 256, 256, 0, s>>>(job.dirty_bricks, job.ndirty, nbricks, mask);
        note_launches(1);
    }
    if (job.ntris) {
        vox_setup<<<uint32_t((job.ntris + 127) / 128), 128, 0, s>>>(job.tri, job.albedo, job.ntris, job.d_frame, dim,
                                                                     sc, d_status);
        vox_bin_big<<<2 * 152, 256, 0, s>>>(dim, sc, d_status, 0);
        note_launches(2);
    }
    int rc = exclusive_scan(sc.brick_count, nbricks, sc.brick_start, sc.total, sc.scan_tmp, s);
    if (rc) return rc;
    if (job.ntris) {
        vox_emit<<<uint32_t((job.ntris + 127) / 128), 128, 0, s>>>(job.ntris, dim, sc, d_status);
        vox_bin_big<<<2 * 152, 256, 0, s>>>(dim, sc, d_status, 1);
        note_launches(2);
    }
    uint32_t nblocks = job.ndirty ? job.ndirty : nbricks;
    vox_bricks<<<nblocks, 256, 0, s>>>(sc, job.d_frame, dim, job.chain, job.light, job.shadow_keys, job.shadow_res,
                                       job.counts, job.ndirty ? job.dirty_bricks : nullptr, d_status);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "voxelize");
}

}  // namespace f184
