// mip.cu -- 3D mip chain of the radiance/opacity grid (2x2x2 mean of premultiplied RGBA).
//
// The reference volume has a single level (Foreground/Renderer/MegaPipeline.cpp:481, Range.Set(0,1,0,1)); this
// pass follows the isotropic pre-filtering of voxel cone tracing (Crassin et al. 2011).  With bricks in Morton
// order, the eight child bricks of a parent brick are contiguous, so one CTA stages a 16^3 source block with a
// single bulk copy (cp.async.bulk + mbarrier) into shared memory and reduces it through up to four levels
// (8^3, 4^3, 2^3, 1) before writing; one pass covers four levels of the chain.
#include "gi_device.cuh"

namespace f184 {
namespace {

constexpr uint32_t kWaitPolls = 1u << 22;

__device__ __forceinline__ float4 raw_vox(const unsigned char* smem, uint32_t format, uint32_t idx) {
    if (format == F184GI_FMT_F32) return reinterpret_cast<const float4*>(smem)[idx];
    uint2 raw = reinterpret_cast<const uint2*>(smem)[idx];
    float2 a = __half22float2(*reinterpret_cast<__half2*>(&raw.x));
    float2 b = __half22float2(*reinterpret_cast<__half2*>(&raw.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4mul(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

// Source block of S^3 voxels of level `src` (S = 16: eight bricks; S <= 8: the whole level) reduced into
// levels src+1 .. src+nout.  Block b of the source level is the Morton-ordered group of 8 bricks 8b .. 8b+7.
__global__ void __launch_bounds__(512) mip_pass(ChainLayout c, uint32_t src, uint32_t nout, uint32_t* status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ float4 lvl[2][512];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t ds = c.ldim[src];
    const uint32_t S = ds >= 16 ? 16u : ds;
    const uint32_t nvox = S * S * S;
    const uint64_t src_off = c.off[src] + (ds >= 16 ? uint64_t(blockIdx.x) * 4096u : 0u);
    const uint32_t bytes = nvox * c.esz;
    const unsigned char* gsrc = static_cast<const unsigned char*>(c.base) + src_off * c.esz;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, bytes);
        bulk_g2s(smem, gsrc, bytes, &bar);
    }
    if (!mbar_wait_bounded(&bar, 0, kWaitPolls)) {
        if (threadIdx.x == 0) set_status(status, kStatusTimeout);
        mbar_wait_bounded(&bar, 0, kWaitPolls);  // let the copy land before the CTA exits
        return;
    }
    // block coordinates of this source block at level src+1 (in units of S/2 voxels)
    uint32_t Bx = 0, By = 0, Bz = 0;
    if (ds >= 16) Bx = compact1by2(blockIdx.x), By = compact1by2(blockIdx.x >> 1), Bz = compact1by2(blockIdx.x >> 2);
    uint32_t n = S / 2;  // output edge of the first produced level
    // level src+1 from the staged source
    const uint32_t t = threadIdx.x;
    if (t < n * n * n) {
        uint32_t x = t % n, y = (t / n) % n, z = t / (n * n);
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    uint32_t sx = 2 * x + dx, sy = 2 * y + dy, sz = 2 * z + dz;
                    uint32_t si;
                    if (S >= 8) {
                        uint32_t cb = ((sx >> 3) & 1u) | (((sy >> 3) & 1u) << 1) | (((sz >> 3) & 1u) << 2);
                        si = cb * 512u + ((sz & 7u) << 6) + ((sy & 7u) << 3) + (sx & 7u);
                    } else {
                        si = (sz * S + sy) * S + sx;
                    }
                    acc = f4add(acc, raw_vox(smem, c.format, si));
                }
        acc = f4mul(acc, 0.125f);
        lvl[0][t] = acc;
        uint32_t d1 = c.ldim[src + 1];
        store_vox(c.base, c.format, c.off[src + 1] + vox_index(d1, Bx * n + x, By * n + y, Bz * n + z), acc);
    }
    __syncthreads();
    int cur = 0;
    for (uint32_t k = 2; k <= nout; ++k) {
        uint32_t np = n;
        n = n / 2;
        if (t < n * n * n) {
            uint32_t x = t % n, y = (t / n) % n, z = t / (n * n);
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int dz = 0; dz < 2; ++dz)
                for (int dy = 0; dy < 2; ++dy)
                    for (int dx = 0; dx < 2; ++dx)
                        acc = f4add(acc, lvl[cur][((2 * z + dz) * np + (2 * y + dy)) * np + (2 * x + dx)]);
            acc = f4mul(acc, 0.125f);
            lvl[cur ^ 1][t] = acc;
            uint32_t dk = c.ldim[src + k];
            store_vox(c.base, c.format, c.off[src + k] + vox_index(dk, Bx * n + x, By * n + y, Bz * n + z), acc);
        }
        __syncthreads();
        cur ^= 1;
    }
}

}  // namespace

int mip_launch(const ChainLayout& c, uint32_t levels, uint32_t* d_status, cudaStream_t s) {
    if (c.aniso) return fail(F184GI_ERR_INVALID, "mip: anisotropic chains are built by mip_aniso_launch");
    if (levels > c.levels) levels = c.levels;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(mip_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16);
        if (e != cudaSuccess) return cuda_fail(e, "mip: smem attribute");
        attr_set = true;
    }
    uint32_t l = 0;
    while (l + 1 < levels) {
        uint32_t ds = c.ldim[l];
        uint32_t S = ds >= 16 ? 16u : ds;
        uint32_t maxout = 0;
        for (uint32_t e = S; e > 1; e /= 2) ++maxout;  // S=16 -> 4 levels
        uint32_t nout = std::min(maxout, levels - 1 - l);
        uint32_t blocks = ds >= 16 ? (ds / 16) * (ds / 16) * (ds / 16) : 1u;
        size_t smem = size_t(S) * S * S * c.esz;
        mip_pass<<<blocks, 512, smem, s>>>(c, l, nout, d_status);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "mip");
        l += nout;
    }
    return F184GI_OK;
}

}  // namespace f184
