// gi_device.cuh -- device helpers shared by the f184gi kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "gi_internal.h"

namespace f184 {

// ---- exact FP64: every operation rounded on its own, never contracted into an FMA ----
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
// row . (x, y, z, 1) in the order ((r0 x + r1 y) + r2 z) + r3
__device__ __forceinline__ double drow(const double* r, double x, double y, double z) {
    double s = dadd(dmul(r[0], x), dmul(r[1], y));
    s = dadd(s, dmul(r[2], z));
    return dadd(s, r[3]);
}

__device__ __forceinline__ int64_t floor_div64(int64_t a, int64_t b) {  // b > 0
    int64_t q = a / b;
    if ((a % b) != 0 && a < 0) --q;
    return q;
}

// ---- Morton order of 8^3 bricks ----
__host__ __device__ __forceinline__ uint32_t part1by2(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
__host__ __device__ __forceinline__ uint32_t compact1by2(uint32_t x) {
    x &= 0x09249249u;
    x = (x | (x >> 2)) & 0x030C30C3u;
    x = (x | (x >> 4)) & 0x0300F00Fu;
    x = (x | (x >> 8)) & 0x030000FFu;
    x = (x | (x >> 16)) & 0x000003FFu;
    return x;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2);
}

// element index of voxel (x, y, z) inside one volume of level `level` with `d` voxels per axis: level 0 is stored
// in 8^3 bricks in Morton order (the voxelizer's unit); coarser levels linearly (x fastest) inside a one-voxel
// ring of zeros, (d + 2)^3 elements, so that every trilinear footprint touching the level is addressable
__host__ __device__ __forceinline__ uint64_t vox_index(uint32_t level, uint32_t d, uint32_t x, uint32_t y,
                                                      uint32_t z) {
    if (level > 0) {
        const uint64_t dp = d + 2;
        return (uint64_t(z + 1) * dp + (y + 1)) * dp + (x + 1);
    }
    if (d >= 8) {
        uint32_t m = morton3(x >> 3, y >> 3, z >> 3);
        return (uint64_t(m) << 9) | ((z & 7u) << 6) | ((y & 7u) << 3) | (x & 7u);
    }
    return (uint64_t(z) * d + y) * d + x;
}

// ---- voxel payload load/store ----
// FP16 chains (8 B a voxel): R, G, B as binary16 and the opacity as 16-bit unorm, n / 65535.  Opacity is what the
// cones composite as transmittance factors 1 - a: binary16 keeps 11 bits relative to a, so near a = 1 the factor
// loses all its precision (a = 0.99 rounds by up to 2.4e-4, 2.4% of 1 - a), while unorm16 keeps 7.6e-6 absolute
// everywhere.  Measured on the anisotropic test chain with the radiance left exact: max relative pixel error
// 1.7e-3 with binary16 opacity, 7e-5 with unorm16 (3.3e-4 with binary16 radiance as well).
constexpr float kUnorm16 = 1.0f / 65535.0f;
__device__ __forceinline__ uint32_t alpha_to_unorm16(float a) {
    return __float2uint_rn(fminf(fmaxf(a, 0.0f), 1.0f) * 65535.0f);
}
__device__ __forceinline__ float4 decode_f16_vox(uint2 raw) {
    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    const float b = __half2float(__ushort_as_half(uint16_t(raw.y & 0xffffu)));
    return make_float4(rg.x, rg.y, b, float(raw.y >> 16) * kUnorm16);
}
__device__ __forceinline__ uint2 encode_f16_vox(float4 v) {
    const __half2 rg = __floats2half2_rn(v.x, v.y);
    uint2 raw;
    raw.x = *reinterpret_cast<const uint32_t*>(&rg);
    raw.y = uint32_t(__half_as_ushort(__float2half_rn(v.z))) | (alpha_to_unorm16(v.w) << 16);
    return raw;
}
__device__ __forceinline__ float4 load_vox(const void* base, uint32_t format, uint64_t idx) {
    if (format == F184GI_FMT_F32) return __ldg(reinterpret_cast<const float4*>(base) + idx);
    return decode_f16_vox(__ldg(reinterpret_cast<const uint2*>(base) + idx));
}
__device__ __forceinline__ void store_vox(void* base, uint32_t format, uint64_t idx, float4 v) {
    if (format == F184GI_FMT_F32) {
        reinterpret_cast<float4*>(base)[idx] = v;
        return;
    }
    reinterpret_cast<uint2*>(base)[idx] = encode_f16_vox(v);
}

// Float-float arithmetic: unevaluated pairs h + l of FP32 (~2^-44 relative), every operation explicitly rounded
// (Knuth's two-sum and the FMA two-product are exact), so a kernel and a restatement compiled without contraction
// that run the same operations get the same bits.
struct FF {
    float h, l;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ FF ff_norm(float s, float e) {  // |s| >= |e|
    const float h = __fadd_rn(s, e);
    return FF{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    return ff_norm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.h, -p)));
    return ff_norm(p, e);
}
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q = __fdiv_rn(a.h, b.h);
    const FF r = ff_add(a, ff_mul(FF{-q, 0.0f}, b));  // a - q b
    return ff_norm(q, __fdiv_rn(r.h, b.h));
}

// The isotropic mip value of a voxel: the mean of its 2x2x2 children, fetch(dx, dy, dz) returning child
// (dx, dy, dz), summed in the order dz, dy, dx (one rounding per add, no multiply feeding an add) and scaled by
// 1/8.  Every kernel that builds an isotropic level calls this, so the chain's bytes do not depend on which one did.
template <class Fetch>
__device__ __forceinline__ float4 iso_mean8(Fetch fetch) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const float4 v = fetch(dx, dy, dz);
                acc = make_float4(acc.x + v.x, acc.y + v.y, acc.z + v.z, acc.w + v.w);
            }
    return make_float4(acc.x * 0.125f, acc.y * 0.125f, acc.z * 0.125f, acc.w * 0.125f);
}

__device__ __forceinline__ void set_status(uint32_t* st, uint32_t bit) {
    if (st) atomicOr(st, bit);
}

// Bounded mbarrier wait on `parity`; returns false (and leaves the barrier) after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(addr) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar` (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
    uint32_t b = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
        "l"(gsrc), "r"(bytes), "r"(b)
        : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

}  // namespace f184
