// mip.cu -- 3D mip chain of the radiance/opacity grid: 2x2x2 mean of premultiplied RGBA (isotropic), or six
// directional volumes per level (anisotropic).
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
    return decode_f16_vox(reinterpret_cast<const uint2*>(smem)[idx]);
}

__device__ __forceinline__ float4 f4mul(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

// One output voxel from its 2x2x2 children, fetch(dx, dy, dz) returning child (dx, dy, dz).
// Isotropic: the mean of the eight children.  Anisotropic direction d in (+x, -x, +y, -y, +z, -z): along the
// axis of d the two children composite front to back (front = the child a cone travelling along d meets first:
// f + (1 - f.alpha) b per channel) and the four columns across the axis are averaged.
template <bool ANISO, class Fetch>
__device__ __forceinline__ float4 reduce8(uint32_t dir, Fetch fetch) {
    if (!ANISO) return iso_mean8(fetch);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const int axis = int(dir >> 1);
    const int neg = int(dir & 1u);
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    for (int u = 0; u < 2; ++u)
        for (int v = 0; v < 2; ++v) {
            int of[3], ob[3];
            of[axis] = neg, ob[axis] = 1 - neg;
            of[o1] = ob[o1] = u;
            of[o2] = ob[o2] = v;
            const float4 f = fetch(of[0], of[1], of[2]);
            const float4 b = fetch(ob[0], ob[1], ob[2]);
            // explicit rounding (one fused multiply-add, then the sum): the same bytes in every kernel that inlines it
            const float tr = __fsub_rn(1.0f, f.w);
            acc.x = __fadd_rn(acc.x, __fmaf_rn(tr, b.x, f.x));
            acc.y = __fadd_rn(acc.y, __fmaf_rn(tr, b.y, f.y));
            acc.z = __fadd_rn(acc.z, __fmaf_rn(tr, b.z, f.z));
            acc.w = __fadd_rn(acc.w, __fmaf_rn(tr, b.w, f.w));
        }
    return f4mul(acc, 0.25f);
}

// Source block of S^3 voxels of level `src` (S = 16, or the whole level when it is smaller) reduced into
// levels src+1 .. src+nout, which are stored linearly inside their zero rings.  Blocks are numbered in Morton
// order of their position.  Level 0 is stored in Morton-ordered 8^3 bricks, so block b is bricks 8b .. 8b+7,
// contiguous: one bulk copy (cp.async.bulk) stages it; a block of a coarser level is gathered row by row.
// Anisotropic chains: CTA x = block * 6 + direction (the six CTAs of one block run together, so a level-0
// block read by all six comes from DRAM once); direction d of a level reduces direction d of the level below
// (level 0 has one volume).
template <bool ANISO>
__global__ void __launch_bounds__(512) mip_pass(ChainLayout c, uint32_t src, uint32_t nout, uint32_t* status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ float4 lvl[2][512];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t dir = ANISO ? blockIdx.x % 6u : 0u;
    const uint32_t blk = ANISO ? blockIdx.x / 6u : blockIdx.x;
    const uint32_t ds = c.ldim[src];
    const uint32_t S = ds >= 16 ? 16u : ds;
    const uint32_t nvox = S * S * S;
    const uint64_t src_vol = (ANISO && src > 0) ? c.off[src] + uint64_t(dir) * c.vol[src] : c.off[src];
    const bool bricked = src == 0;
    // block coordinates of this source block (in blocks of S voxels; at level src+1 in units of S/2 voxels)
    uint32_t Bx = 0, By = 0, Bz = 0;
    if (ds >= 16) Bx = compact1by2(blk), By = compact1by2(blk >> 1), Bz = compact1by2(blk >> 2);
    if (bricked) {
        const uint64_t src_off = src_vol + (ds >= 16 ? uint64_t(blk) * 4096u : 0u);
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
        if (__syncthreads_or(!mbar_wait_bounded(&bar, 0, kWaitPolls))) {  // one branch for the whole CTA
            if (threadIdx.x == 0) {
                set_status(status, kStatusTimeout | kStatusCopyTimeout);
                mbar_wait_bounded(&bar, 0, kWaitPolls);  // let the copy land before the CTA exits (bounded)
            }
            return;
        }
    } else {  // S rows of S x S from the ringed linear level: element e of row (y, z) -> smem (z S + y) S + e
        const unsigned char* gbase = static_cast<const unsigned char*>(c.base);
        for (uint32_t i = threadIdx.x; i < nvox; i += blockDim.x) {
            const uint32_t e = i % S, y = (i / S) % S, z = i / (S * S);
            const uint64_t g = src_vol + vox_index(src, ds, Bx * S + e, By * S + y, Bz * S + z);
            if (c.esz == 16)
                reinterpret_cast<float4*>(smem)[i] = reinterpret_cast<const float4*>(gbase)[g];
            else
                reinterpret_cast<uint2*>(smem)[i] = reinterpret_cast<const uint2*>(gbase)[g];
        }
        __syncthreads();
    }
    uint32_t n = S / 2;  // output edge of the first produced level
    // level src+1 from the staged source
    const uint32_t t = threadIdx.x;
    if (t < n * n * n) {
        const uint32_t x = t % n, y = (t / n) % n, z = t / (n * n);
        const float4 acc = reduce8<ANISO>(dir, [&](int dx, int dy, int dz) {
            const uint32_t sx = 2 * x + dx, sy = 2 * y + dy, sz = 2 * z + dz;
            uint32_t si;
            if (bricked && S >= 8) {
                const uint32_t cb = ((sx >> 3) & 1u) | (((sy >> 3) & 1u) << 1) | (((sz >> 3) & 1u) << 2);
                si = cb * 512u + ((sz & 7u) << 6) + ((sy & 7u) << 3) + (sx & 7u);
            } else {
                si = (sz * S + sy) * S + sx;
            }
            return raw_vox(smem, c.format, si);
        });
        lvl[0][t] = acc;
        const uint32_t d1 = c.ldim[src + 1];
        const uint64_t dst = c.off[src + 1] + (ANISO ? uint64_t(dir) * c.vol[src + 1] : 0u);
        store_vox(c.base, c.format, dst + vox_index(src + 1, d1, Bx * n + x, By * n + y, Bz * n + z), acc);
    }
    __syncthreads();
    int cur = 0;
    for (uint32_t k = 2; k <= nout; ++k) {
        const uint32_t np = n;
        n = n / 2;
        if (t < n * n * n) {
            const uint32_t x = t % n, y = (t / n) % n, z = t / (n * n);
            const float4 acc = reduce8<ANISO>(dir, [&](int dx, int dy, int dz) {
                return lvl[cur][((2 * z + dz) * np + (2 * y + dy)) * np + (2 * x + dx)];
            });
            lvl[cur ^ 1][t] = acc;
            const uint32_t dk = c.ldim[src + k];
            const uint64_t dst = c.off[src + k] + (ANISO ? uint64_t(dir) * c.vol[src + k] : 0u);
            store_vox(c.base, c.format, dst + vox_index(src + k, dk, Bx * n + x, By * n + y, Bz * n + z), acc);
        }
        __syncthreads();
        cur ^= 1;
    }
}

// Isotropic chains, level 0 -> levels 1 .. nout (<= 4), as a stream: one persistent CTA per SM walks the 16^3
// blocks (b = blockIdx.x, += gridDim.x) through a ring of kStages shared-memory buffers, each filled by one bulk
// copy (cp.async.bulk, completion on the buffer's mbarrier).  The copies of the next kStages - 1 blocks are in
// flight while the CTA reduces the current one, so the SM keeps ~2 blocks (128 KB of FP32) of reads outstanding
// instead of none between a block's load and its reduction.  The reductions are mip_pass's, in its order, so the
// bytes are the same.  If a wait expires the CTA records kStatusCopyTimeout, waits (bounded) for every copy it
// still has in flight, and returns.
constexpr uint32_t kStages = 3;
constexpr uint32_t kStageBytes = 4096u * 16u;  // one 16^3 block of FP32 voxels (FP16 blocks use half)

__global__ void __launch_bounds__(512, 1) mip_l0_stream(ChainLayout c, uint32_t nout, uint32_t nblocks,
                                                       uint32_t* status) {
    extern __shared__ __align__(128) unsigned char smem[];  // kStages x kStageBytes
    __shared__ float4 lvl[2][512];
    __shared__ __align__(8) uint64_t bar[kStages];
    const uint32_t t = threadIdx.x;
    const uint32_t bytes = 4096u * c.esz;
    const unsigned char* gbase = static_cast<const unsigned char*>(c.base) + c.off[0] * c.esz;
    if (t == 0) {
        for (uint32_t k = 0; k < kStages; ++k) mbar_init(&bar[k], 1);
        fence_barrier_init();
    }
    __syncthreads();
    uint32_t pending = 0;  // bit k: a copy into stage k is in flight (thread 0's view)
    if (t == 0) {
        for (uint32_t k = 0; k < kStages; ++k) {
            const uint32_t blk = blockIdx.x + k * gridDim.x;
            if (blk >= nblocks) break;
            mbar_expect_tx(&bar[k], bytes);
            bulk_g2s(smem + k * kStageBytes, gbase + uint64_t(blk) * bytes, bytes, &bar[k]);
            pending |= 1u << k;
        }
    }
    const uint32_t d1 = c.ldim[1];
    for (uint32_t i = 0;; ++i) {
        const uint32_t blk = blockIdx.x + i * gridDim.x;
        if (blk >= nblocks) break;
        const uint32_t st = i % kStages;
        const uint32_t parity = (i / kStages) & 1u;
        // every thread waits (bounded); the CTA then takes one branch (a vote), so no barrier below is missed
        if (__syncthreads_or(!mbar_wait_bounded(&bar[st], parity, kWaitPolls))) {
            if (t == 0) {
                set_status(status, kStatusTimeout | kStatusCopyTimeout);
                // let every copy still in flight land before the CTA exits (each wait bounded)
                for (uint32_t k = 0; k < kStages; ++k) {
                    if (!((pending >> k) & 1u)) continue;
                    const uint32_t uses = (k < st) ? (i / kStages) + 1u : (i / kStages);  // waits done on stage k
                    mbar_wait_bounded(&bar[k], uses & 1u, kWaitPolls);
                }
            }
            return;
        }
        if (t == 0) pending &= ~(1u << st);
        const unsigned char* src = smem + st * kStageBytes;
        const uint32_t Bx = compact1by2(blk), By = compact1by2(blk >> 1), Bz = compact1by2(blk >> 2);
        {  // level 1 from the staged block (512 outputs, one per thread)
            const uint32_t x = t % 8u, y = (t / 8u) % 8u, z = t / 64u;
            const float4 acc = reduce8<false>(0u, [&](int dx, int dy, int dz) {
                const uint32_t sx = 2 * x + dx, sy = 2 * y + dy, sz = 2 * z + dz;
                const uint32_t cb = ((sx >> 3) & 1u) | (((sy >> 3) & 1u) << 1) | (((sz >> 3) & 1u) << 2);
                return raw_vox(src, c.format, cb * 512u + ((sz & 7u) << 6) + ((sy & 7u) << 3) + (sx & 7u));
            });
            lvl[0][t] = acc;
            store_vox(c.base, c.format, c.off[1] + vox_index(1, d1, Bx * 8 + x, By * 8 + y, Bz * 8 + z), acc);
        }
        __syncthreads();  // the stage is read: refill it with the block kStages ahead
        if (t == 0) {
            const uint32_t nb = blk + kStages * gridDim.x;
            if (nb < nblocks) {
                mbar_expect_tx(&bar[st], bytes);
                bulk_g2s(smem + st * kStageBytes, gbase + uint64_t(nb) * bytes, bytes, &bar[st]);
                pending |= 1u << st;
            }
        }
        int cur = 0;
        uint32_t n = 8;
        for (uint32_t k = 2; k <= nout; ++k) {
            const uint32_t np = n;
            n = n / 2;
            if (t < n * n * n) {
                const uint32_t x = t % n, y = (t / n) % n, z = t / (n * n);
                const float4 acc = reduce8<false>(0u, [&](int dx, int dy, int dz) {
                    return lvl[cur][((2 * z + dz) * np + (2 * y + dy)) * np + (2 * x + dx)];
                });
                lvl[cur ^ 1][t] = acc;
                store_vox(c.base, c.format,
                          c.off[k] + vox_index(k, c.ldim[k], Bx * n + x, By * n + y, Bz * n + z), acc);
            }
            __syncthreads();
            cur ^= 1;
        }
    }
}

// Anisotropic chains, level 0 -> levels 1 .. nout: level 0 has one volume, so one CTA per 16^3 block stages it
// once (bulk copy) and reduces it along all six directions (six CTAs of mip_pass per block would each stage it);
// each thread keeps its voxel's six level-1 results, which then replace the staged block in shared memory as the
// sources of levels 2 .. nout (per direction, the reductions of mip_pass in its order, hence its bytes).
__global__ void __launch_bounds__(512, 2) mip_aniso_l0(ChainLayout c, uint32_t nout, uint32_t* status) {
    extern __shared__ __align__(128) unsigned char smem[];  // the staged block, then level 1: float4 [6][512]
    __shared__ float4 l2[6 * 64];
    __shared__ float4 l3[6 * 8];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t blk = blockIdx.x;
    const uint32_t Bx = compact1by2(blk), By = compact1by2(blk >> 1), Bz = compact1by2(blk >> 2);
    const uint32_t bytes = 4096u * c.esz;
    const unsigned char* gsrc = static_cast<const unsigned char*>(c.base) + (c.off[0] + uint64_t(blk) * 4096u) * c.esz;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, bytes);
        bulk_g2s(smem, gsrc, bytes, &bar);
    }
    if (__syncthreads_or(!mbar_wait_bounded(&bar, 0, kWaitPolls))) {  // one branch for the whole CTA
        if (threadIdx.x == 0) {
            set_status(status, kStatusTimeout | kStatusCopyTimeout);
            mbar_wait_bounded(&bar, 0, kWaitPolls);  // let the copy land before the CTA exits (bounded)
        }
        return;
    }
    const uint32_t t = threadIdx.x;
    const uint32_t x = t % 8u, y = (t / 8u) % 8u, z = t / 64u;
    float4 acc[6];
#pragma unroll
    for (uint32_t dir = 0; dir < 6; ++dir) {
        acc[dir] = reduce8<true>(dir, [&](int dx, int dy, int dz) {
            const uint32_t sx = 2 * x + dx, sy = 2 * y + dy, sz = 2 * z + dz;
            const uint32_t cb = ((sx >> 3) & 1u) | (((sy >> 3) & 1u) << 1) | (((sz >> 3) & 1u) << 2);
            return raw_vox(smem, c.format, cb * 512u + ((sz & 7u) << 6) + ((sy & 7u) << 3) + (sx & 7u));
        });
        store_vox(c.base, c.format,
                  c.off[1] + uint64_t(dir) * c.vol[1] + vox_index(1, c.ldim[1], Bx * 8 + x, By * 8 + y, Bz * 8 + z),
                  acc[dir]);
    }
    __syncthreads();  // every thread has read the staged block
    float4* l1 = reinterpret_cast<float4*>(smem);
#pragma unroll
    for (uint32_t dir = 0; dir < 6; ++dir) l1[dir * 512 + t] = acc[dir];
    __syncthreads();
    if (nout >= 2 && t < 6 * 64) {
        const uint32_t dir = t / 64u, v = t % 64u, vx = v % 4u, vy = (v / 4u) % 4u, vz = v / 16u;
        const float4 a = reduce8<true>(dir, [&](int dx, int dy, int dz) {
            return l1[dir * 512 + ((2 * vz + dz) * 8 + (2 * vy + dy)) * 8 + (2 * vx + dx)];
        });
        l2[t] = a;
        store_vox(c.base, c.format,
                  c.off[2] + uint64_t(dir) * c.vol[2] + vox_index(2, c.ldim[2], Bx * 4 + vx, By * 4 + vy, Bz * 4 + vz), a);
    }
    __syncthreads();
    if (nout >= 3 && t < 6 * 8) {
        const uint32_t dir = t / 8u, v = t % 8u, vx = v % 2u, vy = (v / 2u) % 2u, vz = v / 4u;
        const float4 a = reduce8<true>(dir, [&](int dx, int dy, int dz) {
            return l2[dir * 64 + ((2 * vz + dz) * 4 + (2 * vy + dy)) * 4 + (2 * vx + dx)];
        });
        l3[t] = a;
        store_vox(c.base, c.format,
                  c.off[3] + uint64_t(dir) * c.vol[3] + vox_index(3, c.ldim[3], Bx * 2 + vx, By * 2 + vy, Bz * 2 + vz), a);
    }
    __syncthreads();
    if (nout >= 4 && t < 6) {
        const uint32_t dir = t;
        const float4 a = reduce8<true>(dir, [&](int dx, int dy, int dz) { return l3[dir * 8 + (dz * 2 + dy) * 2 + dx]; });
        store_vox(c.base, c.format, c.off[4] + uint64_t(dir) * c.vol[4] + vox_index(4, c.ldim[4], Bx, By, Bz), a);
    }
}

uint32_t sm_count_current() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return uint32_t(sms > 0 ? sms : 1);
}

}  // namespace

int mip_launch(const ChainLayout& c, uint32_t levels, uint32_t from, uint32_t* d_status, cudaStream_t s) {
    if (levels > c.levels) levels = c.levels;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(mip_pass<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mip_pass<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mip_aniso_l0, cudaFuncAttributeMaxDynamicSharedMemorySize, 4096 * 16);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(mip_l0_stream, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(kStages * kStageBytes));
        if (e != cudaSuccess) return cuda_fail(e, "mip: smem attribute");
        attr_set = true;
    }
    const uint32_t ndir = c.aniso ? 6u : 1u;
    uint32_t l = from;
    while (l + 1 < levels) {
        uint32_t ds = c.ldim[l];
        uint32_t S = ds >= 16 ? 16u : ds;
        uint32_t maxout = 0;
        for (uint32_t e = S; e > 1; e /= 2) ++maxout;  // S=16 -> 4 levels
        uint32_t nout = std::min(maxout, levels - 1 - l);
        uint32_t blocks = (ds >= 16 ? (ds / 16) * (ds / 16) * (ds / 16) : 1u) * ndir;
        size_t smem = size_t(S) * S * S * c.esz;
        if (c.aniso && l == 0 && ds >= 16)  // one CTA per block for all six directions
            mip_aniso_l0<<<blocks / 6, 512, std::max<size_t>(smem, 6 * 512 * 16), s>>>(c, nout, d_status);
        else if (!c.aniso && l == 0 && ds >= 16)  // the level-0 stream: one persistent CTA per SM
            mip_l0_stream<<<std::min(blocks, sm_count_current()), 512, kStages * kStageBytes, s>>>(c, nout, blocks,
                                                                                               d_status);
        else if (c.aniso)
            mip_pass<true><<<blocks, 512, smem, s>>>(c, l, nout, d_status);
        else
            mip_pass<false><<<blocks, 512, smem, s>>>(c, l, nout, d_status);
        note_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "mip");
        l += nout;
    }
    return F184GI_OK;
}

}  // namespace f184
