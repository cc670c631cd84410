// util.cu -- exclusive scan, scene-bounds reduction + device frame, level read-back.
#include <cfloat>

#include "frame.h"
#include "gi_device.cuh"
#include "util.cuh"

namespace f184 {

// ---------------- exclusive scan of u32 (n <= kScanBlock * kScanBlock) ----------------
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;  // elements per block

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= uint32_t(o)) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= uint32_t(o)) s += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t prefix = wid ? warp_sums[wid - 1] : 0;
    uint32_t tot = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    if (total) *total = tot;
    return prefix + x - v;
}

__global__ void scan_block_sums(const uint32_t* in, uint32_t n, uint32_t* block_sums) {
    uint64_t base = uint64_t(blockIdx.x) * kScanBlock + threadIdx.x * kScanPer;
    uint32_t s = 0;
    for (int i = 0; i < kScanPer; ++i)
        if (base + i < n) s += in[base + i];
    uint32_t tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void scan_top(uint32_t* block_sums, uint32_t nblocks, uint32_t* total_out) {
    // one block: nblocks <= kScanBlock
    uint32_t base = threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
    for (int i = 0; i < kScanPer; ++i) {
        v[i] = base + i < nblocks ? block_sums[base + i] : 0;
        s += v[i];
    }
    uint32_t tot;
    uint32_t pre = block_exclusive_scan(s, &tot);
    for (int i = 0; i < kScanPer; ++i) {
        if (base + i < nblocks) block_sums[base + i] = pre;
        pre += v[i];
    }
    if (threadIdx.x == 0 && total_out) *total_out = tot;
}

__global__ void scan_apply(const uint32_t* in, uint32_t n, const uint32_t* block_sums, uint32_t* out) {
    uint64_t base = uint64_t(blockIdx.x) * kScanBlock + threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
    for (int i = 0; i < kScanPer; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    uint32_t pre = block_exclusive_scan(s, nullptr) + block_sums[blockIdx.x];
    for (int i = 0; i < kScanPer; ++i) {
        if (base + i < n) out[base + i] = pre;
        pre += v[i];
    }
}

}  // namespace

size_t scan_scratch_bytes(uint32_t n) { return (size_t((n + kScanBlock - 1) / kScanBlock) + 1) * 4; }

int exclusive_scan(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* total, void* scratch,
                   cudaStream_t s) {
    uint32_t nblocks = (n + kScanBlock - 1) / kScanBlock;
    if (nblocks == 0) nblocks = 1;
    if (nblocks > uint32_t(kScanBlock)) return fail(F184GI_ERR_INVALID, "scan: too many elements");
    uint32_t* bs = static_cast<uint32_t*>(scratch);
    scan_block_sums<<<nblocks, kScanThreads, 0, s>>>(in, n, bs);
    scan_top<<<1, kScanThreads, 0, s>>>(bs, nblocks, total);
    scan_apply<<<nblocks, kScanThreads, 0, s>>>(in, n, bs, out);
    note_launches(3);
    return cuda_fail(cudaGetLastError(), "scan");
}

// ---------------- bounds + device frame ----------------
namespace {

__device__ __forceinline__ int32_t ordered(float f) {
    int32_t i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unordered(int32_t i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void bounds_init(int32_t* mm) {
    if (threadIdx.x < 3) {
        mm[threadIdx.x] = ordered(FLT_MAX);
        mm[3 + threadIdx.x] = ordered(-FLT_MAX);
    }
}

__global__ void bounds_reduce(const float* tri, uint64_t nfloats, int32_t* mm) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    uint64_t stride = uint64_t(gridDim.x) * blockDim.x * 3;
    for (uint64_t i = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * 3; i + 2 < nfloats; i += stride)
        for (int a = 0; a < 3; ++a) {
            float v = tri[i + a];
            mn[a] = fminf(mn[a], v);
            mx[a] = fmaxf(mx[a], v);
        }
    for (int a = 0; a < 3; ++a)
        for (int o = 16; o; o >>= 1) {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; ++a) {
            atomicMin(&mm[a], ordered(mn[a]));
            atomicMax(&mm[3 + a], ordered(mx[a]));
        }
}

__global__ void frame_kernel(const int32_t* mm, f184gi_bounds bounds, int use_mm, uint32_t dim, float lx, float ly,
                             float lz, f184gi_grid_frame* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float mn[3] = {bounds.min.x, bounds.min.y, bounds.min.z}, mx[3] = {bounds.max.x, bounds.max.y, bounds.max.z};
    if (use_mm)
        for (int a = 0; a < 3; ++a) {
            mn[a] = unordered(mm[a]);
            mx[a] = unordered(mm[3 + a]);
        }
    const float L[3] = {lx, ly, lz};
    frame_from_bounds(mn, mx, dim, L, out);
    // the voxel map as FP32 pairs, after the frame (the trace's FP64-free set-up)
    FramePairs* fp = reinterpret_cast<FramePairs*>(out + 1);
    for (int a = 0; a < 3; ++a) {
        fp->org_h[a] = __double2float_rn(out->origin[a]);
        fp->org_l[a] = __double2float_rn(__dsub_rn(out->origin[a], double(fp->org_h[a])));
    }
    const double ivs = __dmul_rn(out->inv_voxel_fixed, 1.0 / 256.0);
    fp->ivs_h = __double2float_rn(ivs);
    fp->ivs_l = __double2float_rn(__dsub_rn(ivs, double(fp->ivs_h)));
}

// The frame block computed on the host, passed by value and stored by one warp.
__global__ void frame_store(FrameBlock fb, f184gi_grid_frame* out) {
    constexpr uint32_t kWords = uint32_t(sizeof(FrameBlock) / 4);
    static_assert(sizeof(FrameBlock) % 4 == 0, "whole words");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&fb);
    uint32_t* dst = reinterpret_cast<uint32_t*>(out);
    for (uint32_t i = threadIdx.x; i < kWords; i += blockDim.x) dst[i] = src[i];
}

}  // namespace

int frame_launch(const float* tri, uint64_t ntris, const f184gi_bounds* bounds, uint32_t dim,
                 const float light_dir[3], f184gi_grid_frame* d_frame, void* scratch, cudaStream_t s) {
    int32_t* mm = static_cast<int32_t*>(scratch);
    f184gi_bounds b{};
    if (!bounds) {
        bounds_init<<<1, 32, 0, s>>>(mm);
        uint64_t nthreads = ntris;
        uint32_t blocks = uint32_t(std::min<uint64_t>((nthreads + 255) / 256, 152 * 8));
        if (blocks == 0) blocks = 1;
        bounds_reduce<<<blocks, 256, 0, s>>>(tri, ntris * 9, mm);
        note_launches(2);
    } else {
        // Given bounds: the frame on the host (the same bytes as the device kernel, which is one thread of FP64
        // work on the critical path of a voxelization), stored by a kernel that takes it as its argument.
        FrameBlock fb;
        int rc = compute_frame_block(*bounds, dim, light_dir, &fb);
        if (rc) return rc;
        frame_store<<<1, 32, 0, s>>>(fb, d_frame);
        note_launches(1);
        return cuda_fail(cudaGetLastError(), "frame");
    }
    frame_kernel<<<1, 32, 0, s>>>(mm, b, 1, dim, light_dir[0], light_dir[1], light_dir[2], d_frame);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "frame");
}

// ---------------- level read-back (level layout -> linear FP32) ----------------
namespace {
__global__ void read_level_kernel(ChainLayout c, uint32_t level, uint32_t dir, float4* out) {
    uint32_t d = c.ldim[level];
    uint64_t n = uint64_t(d) * d * d;
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x = uint32_t(i % d), y = uint32_t((i / d) % d), z = uint32_t(i / (uint64_t(d) * d));
    uint64_t e = c.off[level] + uint64_t(dir) * c.vol[level] + vox_index(level, d, x, y, z);
    out[i] = load_vox(c.base, c.format, e);
}
}  // namespace

int read_level_launch(const ChainLayout& c, uint32_t level, uint32_t dir, float* d_out, cudaStream_t s) {
    uint64_t d = c.ldim[level];
    uint64_t n = d * d * d;
    read_level_kernel<<<uint32_t((n + 255) / 256), 256, 0, s>>>(c, level, dir, reinterpret_cast<float4*>(d_out));
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "read_level");
}

}  // namespace f184

// ---------------- instance transform (tc::Matrix3x4 applied to object-space triangles) ----------------
namespace f184 {
namespace {
struct Mat34 {
    float m[12];
};
__global__ void transform_kernel(const float* __restrict__ src, uint64_t nverts, Mat34 M, float* __restrict__ dst) {
    uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= nverts) return;
    float x = src[v * 3], y = src[v * 3 + 1], z = src[v * 3 + 2];
    for (int r = 0; r < 3; ++r)
        dst[v * 3 + r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M.m[r * 4], x), __fmul_rn(M.m[r * 4 + 1], y)),
                                             __fmul_rn(M.m[r * 4 + 2], z)),
                                   M.m[r * 4 + 3]);
}
}  // namespace

int transform_launch(const float* src, uint64_t ntris, const float model[12], float* dst, cudaStream_t s) {
    Mat34 M;
    for (int i = 0; i < 12; ++i) M.m[i] = model[i];
    uint64_t nv = ntris * 3;
    if (nv == 0) return F184GI_OK;
    transform_kernel<<<uint32_t((nv + 255) / 256), 256, 0, s>>>(src, nv, M, dst);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "transform");
}
}  // namespace f184

// ---------------- rigid moves of triangle ranges ----------------
namespace f184 {
namespace {
constexpr int kMovesPerLaunch = 64;
struct MoveTable {
    f184gi_move m[kMovesPerLaunch];
    uint32_t start[kMovesPerLaunch + 1];  // prefix of vertex counts
    uint32_t n;
};
__global__ void moves_kernel(float* __restrict__ tri, MoveTable t) {
    const uint32_t total = t.start[t.n];
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < total; v += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = t.n;
        while (hi - lo > 1) {
            uint32_t mid = (lo + hi) / 2;
            if (t.start[mid] <= v) lo = mid; else hi = mid;
        }
        const f184gi_move& m = t.m[lo];
        const uint64_t vert = uint64_t(m.first) * 3 + (v - t.start[lo]);
        for (int a = 0; a < 3; ++a) tri[vert * 3 + a] = __fadd_rn(tri[vert * 3 + a], m.offset[a]);
    }
}
}  // namespace

namespace {
// One bounded wait on a shared-memory mbarrier whose phase completes only if `complete` (one arrival); on expiry
// the status word gets the timeout bit, as the library's own bounded waits (the mip pass's bulk-copy wait) do.
__global__ void bounded_wait_selftest(uint32_t polls, uint32_t complete, uint32_t* status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (complete == 1 && threadIdx.x == 0) mbar_arrive(&bar);
    const bool done = mbar_wait_bounded(&bar, 0, polls);
    if (!done && threadIdx.x == 0) set_status(status, kStatusTimeout | (complete == 2 ? kStatusCopyTimeout : 0u));
}
}  // namespace

int bounded_wait_selftest_launch(uint32_t polls, uint32_t complete, uint32_t* status, cudaStream_t s) {
    bounded_wait_selftest<<<1, 32, 0, s>>>(polls, complete, status);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "bounded wait self-test");
}

int moves_launch(float* tri, const f184gi_move* moves, uint32_t nmoves, cudaStream_t s) {
    for (uint32_t b = 0; b < nmoves; b += kMovesPerLaunch) {
        MoveTable t{};
        t.n = std::min<uint32_t>(kMovesPerLaunch, nmoves - b);
        t.start[0] = 0;
        for (uint32_t i = 0; i < t.n; ++i) {
            t.m[i] = moves[b + i];
            t.start[i + 1] = t.start[i] + moves[b + i].count * 3;
        }
        if (t.start[t.n] == 0) continue;
        moves_kernel<<<std::min<uint32_t>((t.start[t.n] + 255) / 256, 152 * 4), 256, 0, s>>>(tri, t);
        note_launches(1);
    }
    return cuda_fail(cudaGetLastError(), "apply_moves");
}
}  // namespace f184
