#pragma once
// trace_kernel.cuh -- the cone-trace kernel: per-pixel diffuse + specular cones over a G-buffer.
//
// Replaces the reference's indirect pass (Shader/Lighting/indirect.frag:104-243), which marches four
// stochastic single rays per pixel through a one-level RG16UI volume.  Here each pixel traces five diffuse cones
// (60-degree aperture: one along the normal, four tilted 60 degrees, in the frame of the reference's
// make_coord_space, indirect.frag:71-86) and one specular cone whose tan(half aperture) is the G-buffer
// roughness.  A cone steps by half its diameter, samples the mip chain quadrilinearly (trilinear inside a
// level, linear between log2(diameter) levels, zero outside the grid) and composites front to back in FP32.
// The G-buffer decode follows indirect.frag:44-58 and 189-196 (InvProj, then InvModelView).
#include "gi_device.cuh"

namespace f184 {
namespace {

// Vector helpers with every operation rounded on its own (the intrinsics are never contracted into FMAs): the
// per-pixel set-up then computes the same bits in every kernel variant, however each is scheduled, and the same
// bits as the FP32 restatement, which is compiled without contraction.
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) {
    return f3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
    return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float3 mul3(float3 a, float s) {
    return f3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
// acc += w * v per component as two packed FP32 FMAs (fma.rn.f32x2): each component is rounded once, exactly
// as fmaf(w, v.c, acc.c), with half the instructions.
__device__ __forceinline__ unsigned long long pack2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ void fma4(float4& acc, float w, const float4& v) {
    const unsigned long long ww = pack2(w, w);
    unsigned long long lo, hi;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(lo) : "l"(ww), "l"(pack2(v.x, v.y)), "l"(pack2(acc.x, acc.y)));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(hi) : "l"(ww), "l"(pack2(v.z, v.w)), "l"(pack2(acc.z, acc.w)));
    unpack2(lo, acc.x, acc.y);
    unpack2(hi, acc.z, acc.w);
}
__device__ __forceinline__ float3 norm3(float3 a) {
    float l = __fsqrt_rn(dot3(a, a));
    return l > 0.0f ? mul3(a, __fdiv_rn(1.0f, l)) : a;
}

// make_coord_space, indirect.frag:71-86
__device__ __forceinline__ void coord_space(float3 n, float3& x, float3& y, float3& z) {
    z = n;
    float3 h = z;
    float ax = fabsf(h.x), ay = fabsf(h.y), az = fabsf(h.z);
    if (ax <= ay && ax <= az)
        h.x = 1.0f;
    else if (ay <= ax && ay <= az)
        h.y = 1.0f;
    else
        h.z = 1.0f;
    z = norm3(z);
    y = norm3(cross3(h, z));
    x = norm3(cross3(z, y));
}

__device__ __forceinline__ float3 oct_decode(uint32_t p) {
    float x = __half2float(__ushort_as_half(uint16_t(p & 0xffffu)));
    float y = __half2float(__ushort_as_half(uint16_t(p >> 16)));
    float3 v = f3(x, y, __fsub_rn(__fsub_rn(1.0f, fabsf(x)), fabsf(y)));
    if (v.z < 0.0f) {
        float ox = v.x, oy = v.y;
        v.x = __fmul_rn(__fsub_rn(1.0f, fabsf(oy)), ox >= 0.0f ? 1.0f : -1.0f);
        v.y = __fmul_rn(__fsub_rn(1.0f, fabsf(ox)), oy >= 0.0f ? 1.0f : -1.0f);
    }
    return norm3(v);
}

// Address of element `idx` of a chain and the voxel `k` elements further (k an immediate offset of the load).
template <int FMT>
__device__ __forceinline__ const unsigned char* vox_ptr(const void* base, uint32_t idx) {
    return static_cast<const unsigned char*>(base) + size_t(idx) * (FMT == F184GI_FMT_F32 ? 16u : 8u);
}
// FP16 chains: the opacity comes back as its unorm16 integer n (not n / 65535); the cone scales its opacity sum
// once per step (kAlphaScale), so a tap costs one conversion per channel as with binary16.
template <int FMT>
__device__ __forceinline__ float4 load_vox_at(const unsigned char* p, int k) {
    if (FMT == F184GI_FMT_F32) return __ldg(reinterpret_cast<const float4*>(p) + k);
    const uint2 raw = __ldg(reinterpret_cast<const uint2*>(p) + k);
    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    const float b = __half2float(__ushort_as_half(uint16_t(raw.y & 0xffffu)));
    return make_float4(rg.x, rg.y, b, float(raw.y >> 16));
}
template <int FMT>
__device__ __forceinline__ float4 load_vox_raw(const void* base, uint32_t idx) {
    return load_vox_at<FMT>(static_cast<const unsigned char*>(base) + size_t(idx) * (FMT == F184GI_FMT_F32 ? 16u : 8u), 0);
}
template <int FMT>
constexpr float kAlphaScale = FMT == F184GI_FMT_F32 ? 1.0f : kUnorm16;

// The pixel set-up runs in float-float arithmetic (FF, gi_device.cuh).  The cone origin in voxel units comes out
// accurate to ~1e-9 voxel; an FP32 set-up (~1e-5 voxel at 256 voxels) moves the trilinear weights of a grazing
// cone's first samples by 1e-5, which is a relative error of 1e-2 on a sample weighted 1e-3.
// (h[0..3] + l[0..3]) . (x, y, z, 1)
__device__ __forceinline__ FF ff_row(const float* h, const float* l, FF x, FF y, FF z) {
    FF s = ff_add(ff_mul(FF{h[0], l[0]}, x), ff_mul(FF{h[1], l[1]}, y));
    s = ff_add(s, ff_mul(FF{h[2], l[2]}, z));
    return ff_add(s, FF{h[3], l[3]});
}
// (2 k + 1) / n - 1: the normalised device coordinate of pixel k of n
__device__ __forceinline__ FF ff_ndc(uint32_t k, uint32_t n) {
    const float num = float(2u * k + 1u), den = float(n);  // exact: n <= 16384
    const float q = __fdiv_rn(num, den);
    const float ql = __fdiv_rn(__fmaf_rn(-q, den, num), den);
    return ff_add(FF{q, ql}, FF{-1.0f, 0.0f});
}

// The grid a warp's tile traces against, staged in shared memory per warp: lanes index the level table with their
// own (divergent) level, which the constant bank would serialise, and batched launches trace many grids.
struct GridRef {
    uint32_t off[kMaxLevels];  // element offsets (a chain holds < 2^32 elements: dim <= 512)
    uint32_t vol[kMaxLevels];
    const void* base;
    uint32_t dim, levels;
    float tmax;
    float org_h[3], org_l[3];  // world -> L0 voxel units: (p - origin) * inv_vs, as float-float pairs
    float ivs_h, ivs_l;
};

// Brick-offset table staged in shared memory: lut[a * kLut + b] = part1by2(b) << (9 + a), the element offset of
// brick coordinate b along axis a (b <= 64 covers dim 512).  The brick offset of (bx, by, bz) is the sum of
// three entries, and the step to the next brick along an axis is the difference of two.
constexpr int kLut = 65;

// 8-tap trilinear sample of one volume of level l (d voxels per axis) at the sample point (L0 voxel units); taps
// outside the volume read zero.  Levels >= 1 are linear inside a ring of zeros: a footprint that touches the volume
// is read whole with deltas +1 / +(d+2) / +(d+2)^2, any other is zero.  Level 0 is bricked: interior samples
// address the seven other taps from the first one with +1 / +8 / +64 inside a brick, or the Morton step to the next
// brick when the tap crosses a brick face; samples touching its border test each tap.
// The sample is ADDED to acc scaled by `scale` (the weight of this level in the quadrilinear blend), which is
// folded into the z weights: acc += scale * sum_taps w_tap v_tap.
template <int FMT, int NV, bool COARSE = false>
__device__ __forceinline__ void tri_sample(const void* base, int d, uint32_t l, const uint32_t (&vol_off)[NV],
                                          float3 oi, float3 xr, const uint32_t* lut, float scale,
                                          float4 (&acc)[NV]) {
    // NV volumes of the same level share the tap coordinates and weights (the three directions an anisotropic
    // sample blends); each volume accumulates its own taps in the single-volume order.
    // The sample point is oi + xr (oi integer, xr small).  Level l's coordinate is u = (oi + xr) 2^-l - 0.5.  At
    // level 0 the tap fraction must keep the precision of xr (a grazing cone's first samples: the FP32 sum oi + xr
    // alone costs 7e-3 relative error on a 512^3 view), so u is split exactly as (oi - 1) + (xr + 0.5).  Coarser
    // levels scale the rounding of p = oi + xr (FP32) by 2^-l and take u + 1 = p 2^-l + 0.5 in FP32, whose floor is
    // the footprint's first voxel in the ringed volume (measured in the FP32 restatement against the split at
    // every level: the same maximum error on the 256^3 plain-large and the 512^3 anisotropic views).
    const float oa[3] = {oi.x, oi.y, oi.z}, xa[3] = {xr.x, xr.y, xr.z};
    int c0[3];
    float f[3];
    if (COARSE || l > 0) {  // COARSE: the caller knows l >= 1 (the level-0 paths are not compiled)
        const float sc = __int_as_float((127 - int(l)) << 23);  // 2^-l
        int c1[3];  // c0 + 1: the footprint's first voxel in the ringed volume
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float u = __fmaf_rn(__fadd_rn(oa[a], xa[a]), sc, 0.5f);
            const float fl = floorf(u);
            c1[a] = int(fl);
            f[a] = __fsub_rn(u, fl);
        }
        // ringed linear level: footprints that touch the volume are read whole (the ring reads zero), the others
        // are zero outright
        if (unsigned(c1[0]) > unsigned(d) || unsigned(c1[1]) > unsigned(d) || unsigned(c1[2]) > unsigned(d))
            return;
        const float wx[2] = {1.0f - f[0], f[0]}, wy[2] = {1.0f - f[1], f[1]};
        const float wz[2] = {(1.0f - f[2]) * scale, f[2] * scale};
        // one address per x-row of the footprint: the row's second tap is the next element (an immediate offset)
        const uint32_t dp = uint32_t(d) + 2u;
        const uint32_t i0 = (uint32_t(c1[2]) * dp + uint32_t(c1[1])) * dp + uint32_t(c1[0]);
        const uint32_t ry = dp, rz = dp * dp;
#pragma unroll
        for (int tz = 0; tz < 2; ++tz)
#pragma unroll
            for (int ty = 0; ty < 2; ++ty) {
                const float wyz = wy[ty] * wz[tz];
                const uint32_t row = i0 + (tz ? rz : 0u) + (ty ? ry : 0u);
                const float w0 = wx[0] * wyz, w1 = wx[1] * wyz;
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    const unsigned char* pr = vox_ptr<FMT>(base, vol_off[k] + row);
                    fma4(acc[k], w0, load_vox_at<FMT>(pr, 0));
                    fma4(acc[k], w1, load_vox_at<FMT>(pr, 1));
                }
            }
        return;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float v = __fadd_rn(xa[a], 0.5f);
        const float fl = floorf(v);
        c0[a] = int(__fadd_rn(__fsub_rn(oa[a], 1.0f), fl));
        f[a] = __fsub_rn(v, fl);
    }
    const float wx[2] = {1.0f - f[0], f[0]}, wy[2] = {1.0f - f[1], f[1]};
    const float wz[2] = {(1.0f - f[2]) * scale, f[2] * scale};
    const unsigned lim = unsigned(d - 1);
    if (unsigned(c0[0]) < lim && unsigned(c0[1]) < lim && unsigned(c0[2]) < lim) {
        uint32_t i0, dx, dy, dz;
        if (d >= 8) {  // level 0: Morton-ordered bricks
            const uint32_t bx = uint32_t(c0[0]) >> 3, by = uint32_t(c0[1]) >> 3, bz = uint32_t(c0[2]) >> 3;
            const uint32_t hx = lut[bx], hy = lut[kLut + by], hz = lut[2 * kLut + bz];
            i0 = hx + hy + hz + ((uint32_t(c0[2] & 7) << 6) | (uint32_t(c0[1] & 7) << 3) | uint32_t(c0[0] & 7));
            // crossing the brick face: local coordinate 7 -> 0 and the brick offset steps along the axis
            dx = (c0[0] & 7) != 7 ? 1u : lut[bx + 1] - hx - 7u;
            dy = (c0[1] & 7) != 7 ? 8u : lut[kLut + by + 1] - hy - 56u;
            dz = (c0[2] & 7) != 7 ? 64u : lut[2 * kLut + bz + 1] - hz - 448u;
        } else {
            i0 = (uint32_t(c0[2]) * uint32_t(d) + uint32_t(c0[1])) * uint32_t(d) + uint32_t(c0[0]);
            dx = 1u, dy = uint32_t(d), dz = uint32_t(d) * uint32_t(d);
        }
#pragma unroll
        for (int tz = 0; tz < 2; ++tz)
#pragma unroll
            for (int ty = 0; ty < 2; ++ty) {
                const float wyz = wy[ty] * wz[tz];
                const uint32_t row = i0 + (tz ? dz : 0u) + (ty ? dy : 0u);
#pragma unroll
                for (int tx = 0; tx < 2; ++tx) {
                    const float w = wx[tx] * wyz;
                    const uint32_t e = row + (tx ? dx : 0u);
#pragma unroll
                    for (int k = 0; k < NV; ++k) {
                        const float4 v = load_vox_raw<FMT>(base, vol_off[k] + e);
                        fma4(acc[k], w, v);
                    }
                }
            }
        return;
    }
    // border: per-axis validity, high (Morton) and low (in-brick / linear) address parts
    bool ok[3][2];
    uint32_t hi[3][2], lo[3][2];
    const bool bricked = d >= 8;  // level 0 only
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            int c = c0[a] + t;
            ok[a][t] = unsigned(c) < unsigned(d);
            uint32_t cu = uint32_t(c) & 1023u;
            if (bricked) {
                hi[a][t] = part1by2(cu >> 3) << a;
                lo[a][t] = (cu & 7u) << (3 * a);
            } else {
                hi[a][t] = 0;
                lo[a][t] = a == 0 ? cu : (a == 1 ? cu * uint32_t(d) : cu * uint32_t(d * d));
            }
        }
#pragma unroll
    for (int tz = 0; tz < 2; ++tz)
#pragma unroll
        for (int ty = 0; ty < 2; ++ty) {
            const float wyz = wy[ty] * wz[tz];
#pragma unroll
            for (int tx = 0; tx < 2; ++tx) {
                if (ok[0][tx] && ok[1][ty] && ok[2][tz]) {
                    const uint32_t idx =
                        ((hi[0][tx] | hi[1][ty] | hi[2][tz]) << 9) | (lo[0][tx] | lo[1][ty] | lo[2][tz]);
                    const float w = wx[tx] * wyz;
#pragma unroll
                    for (int k = 0; k < NV; ++k) {
                        const float4 v = load_vox_raw<FMT>(base, vol_off[k] + idx);
                        fma4(acc[k], w, v);
                    }
                }
            }
        }
}

// acc += scale * (the sample of level l at x): isotropic, or the three direction volumes facing the cone
// weighted by dir^2 (anisotropic levels >= 1)
template <int FMT, bool ANISO, bool COARSE = false>
__device__ __forceinline__ void level_sample(const GridRef& g, const uint32_t* lut, uint32_t l, float3 oi,
                                             float3 x, float3 dir, float scale, float4& acc) {
    const int d = int(g.dim >> l);
    if (!ANISO || l == 0) {
        const uint32_t vo[1] = {g.off[l]};
        float4 a[1] = {acc};
        tri_sample<FMT, 1, COARSE>(g.base, d, l, vo, oi, x, lut, scale, a);
        acc = a[0];
        return;
    }
    const float w[3] = {dir.x * dir.x * scale, dir.y * dir.y * scale, dir.z * dir.z * scale};
    const uint32_t vo[3] = {g.off[l] + (dir.x >= 0.0f ? 0u : 1u) * g.vol[l],
                            g.off[l] + (dir.y >= 0.0f ? 2u : 3u) * g.vol[l],
                            g.off[l] + (dir.z >= 0.0f ? 4u : 5u) * g.vol[l]};
    float4 sa[3] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    tri_sample<FMT, 3, COARSE>(g.base, d, l, vo, oi, x, lut, 1.0f, sa);
#pragma unroll
    for (int a = 0; a < 3; ++a) fma4(acc, w[a], sa[a]);
}

// sched: the first ns samples of this cone's march (the diffuse schedule; ns = 0 for the specular cone).
// COUNT (the instrumented kernel): cnt[0] += steps, cnt[1] += level samples.
template <int FMT, bool ANISO, bool COUNT>
__device__ float4 cone(const GridRef& g, const uint32_t* lut, const TraceConsts& tc, float3 oi, float3 of, float3 dir,
                       float tan_half, const SchedEntry* sched, uint32_t ns, uint32_t* cnt) {
    float cr = 0.f, cg = 0.f, cb = 0.f, alpha = 0.f;
    // The march distance is the float pair t + tl, advanced with error-free sums: a cone of small aperture takes
    // a hundred steps much shorter than t, and plain FP32 sums would drift by ~n/2 ulp(t) (5e-3 voxel at the far
    // end of a 512^3 grid), enough to move samples across opacity edges.
    float t = tc.p.start_offset, tl = 0.0f;
    // the grid's scalars in registers for the whole march: every shared-memory read is a load-pipe wavefront, and
    // the kernel's load pipe is as busy as its issue slots
    const uint32_t gdim = g.dim, glevels = g.levels;
    const float gtmax = g.tmax;
    const float dimf = float(gdim);
    const float maxl = float(glevels - 1);
    const float d2 = 2.0f * tan_half;
    // The exit test (a sample more than 2 diameters outside the grid reads zero, so the cone stops there) can
    // only fire for a cone that starts outside the grid or outruns the margin: the margin 2 diam = 4 t tan grows
    // faster than the distance t travelled once tan >= 0.25, so a cone starting inside with tan >= 0.3 (the
    // diffuse cones' 0.577 and wide specular cones) never meets it and skips it.
    const float3 o0 = add3(oi, of);
    const bool exit_test = !(tan_half >= 0.3f && o0.x >= 0.0f && o0.y >= 0.0f && o0.z >= 0.0f && o0.x <= dimf &&
                             o0.y <= dimf && o0.z <= dimf);
    for (uint32_t k = 0;; ++k) {
        float diam, lraw;
        if (k < ns) {
            const SchedEntry e = sched[k];
            t = e.t, tl = e.tl, diam = e.diam, lraw = e.lvl;
        } else {
            diam = fmaxf(1.0f, fmaf(d2, t, d2 * tl));
            lraw = fmaxf(log2f(diam), 0.0f);
        }
        if (!(t < gtmax || (t == gtmax && tl <= 0.0f))) break;
        float lvl = fminf(lraw, maxl);
        // the sample point oi + x: x is the offset from the origin's integer voxel (small near the surface, where
        // the weights of a grazing cone are most sensitive)
        float3 x = f3(fmaf(dir.x, t, fmaf(dir.x, tl, of.x)), fmaf(dir.y, t, fmaf(dir.y, tl, of.y)),
                      fmaf(dir.z, t, fmaf(dir.z, tl, of.z)));
        if (exit_test) {
            const float m = 2.0f * diam;
            const float3 p = add3(oi, x);
            if (p.x < -m || p.y < -m || p.z < -m || p.x > dimf + m || p.y > dimf + m || p.z > dimf + m) break;
        }
        float fl = floorf(lvl);
        uint32_t l0 = uint32_t(fl);
        float f = lvl - fl;
        if constexpr (COUNT) {
            cnt[0] += 1u;
            cnt[1] += (f > 0.0f && l0 + 1 < glevels) ? 2u : 1u;
        }
        // quadrilinear: (1 - f) * level l0 + f * level l0 + 1, the level weights folded into the tap weights
        const bool two = f > 0.0f && l0 + 1 < glevels;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        level_sample<FMT, ANISO>(g, lut, l0, oi, x, dir, two ? 1.0f - f : 1.0f, s);
        // the finer level's neighbour above is never level 0: its copy carries the ringed path only
        if (two) level_sample<FMT, ANISO, true>(g, lut, l0 + 1, oi, x, dir, f, s);
        if (FMT != F184GI_FMT_F32) s.w *= kAlphaScale<FMT>;  // the unorm16 opacity sum, scaled once
        // front-to-back composite, one fused multiply-add per channel (explicit: the same rounding in every variant)
        const float tr = __fsub_rn(1.0f, alpha);
        cr = __fmaf_rn(tr, s.x, cr);
        cg = __fmaf_rn(tr, s.y, cg);
        cb = __fmaf_rn(tr, s.z, cb);
        alpha = __fmaf_rn(tr, s.w, alpha);
        if (alpha >= tc.p.alpha_stop) break;
        if (k + 1 >= ns) {
            // error-free sum t + step (explicit rounding: no contraction of the step's product into the sum)
            const float step = __fmul_rn(tc.p.step_factor, diam);
            const float ts = __fadd_rn(t, step), tb = __fsub_rn(ts, t);
            tl = __fadd_rn(tl, __fadd_rn(__fsub_rn(t, __fsub_rn(ts, tb)), __fsub_rn(step, tb)));
            t = ts;
        }
    }
    return make_float4(cr, cg, cb, alpha);
}

__device__ __forceinline__ void store_out(void* out, uint32_t fmt, uint64_t i, float4 v) {
    if (fmt == F184GI_FMT_F32) {
        reinterpret_cast<float4*>(out)[i] = v;
    } else {
        __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
        uint2 raw;
        raw.x = *reinterpret_cast<uint32_t*>(&a);
        raw.y = *reinterpret_cast<uint32_t*>(&b);
        reinterpret_cast<uint2*>(out)[i] = raw;
    }
}

template <int FMT, bool ANISO, bool COUNT>
__device__ void trace_pixel(const GridRef& g, const uint32_t* lut, const TraceConsts& tc, const TraceView& v,
                            uint32_t px, uint32_t py, const SchedEntry* sched, uint32_t* cnt) {
    const uint64_t npix = uint64_t(v.width) * v.height;
    const uint64_t pi = uint64_t(py) * v.width + px;
    float d = v.depth[pi];
    if (!(d < 1.0f)) {
        store_out(v.out, v.out_format, pi, make_float4(0.f, 0.f, 0.f, 0.f));
        store_out(v.out, v.out_format, npix + pi, make_float4(0.f, 0.f, 0.f, 0.f));
        return;
    }
    const float* iv = v.iview;
    // View-space and world position in float-float: clip (ndc x, ndc y, depth, 1) through the FP64 inverse
    // projection (rows as FP32 pairs), the perspective division, then the inverse view (rows as FP32 pairs).
    const FF ndx = ff_ndc(px, v.width), ndy = ff_ndc(py, v.height), dz = FF{d, 0.0f};
    const FF vw = ff_row(v.iproj_h + 12, v.iproj_l + 12, ndx, ndy, dz);
    const FF cx = ff_div(ff_row(v.iproj_h, v.iproj_l, ndx, ndy, dz), vw);
    const FF cy = ff_div(ff_row(v.iproj_h + 4, v.iproj_l + 4, ndx, ndy, dz), vw);
    const FF cz = ff_div(ff_row(v.iproj_h + 8, v.iproj_l + 8, ndx, ndy, dz), vw);
    FF wpf[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) wpf[r] = ff_row(v.iview_h + 4 * r, v.iview_l + 4 * r, cx, cy, cz);
    const float3 wp = f3(wpf[0].h, wpf[1].h, wpf[2].h);
    float3 nv = oct_decode(v.normal[pi]);
    float3 nw = norm3(f3(dot3(f3(iv[0], iv[1], iv[2]), nv), dot3(f3(iv[4], iv[5], iv[6]), nv),
                         dot3(f3(iv[8], iv[9], iv[10]), nv)));
    float rough = __half2float(__ushort_as_half(v.rough[pi]));
    // cone origin o = (wp - origin) * inv_vs + n * start_offset in voxel units, split as oi (integer) + of
    float3 oi, of;
    {
        const float na[3] = {nw.x, nw.y, nw.z};
        float oia[3], ofa[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const FF pv = ff_mul(ff_add(wpf[a], FF{-g.org_h[a], -g.org_l[a]}), FF{g.ivs_h, g.ivs_l});
            const float q = __fmul_rn(na[a], tc.p.start_offset);
            const FF o = ff_add(pv, FF{q, __fmaf_rn(na[a], tc.p.start_offset, -q)});
            oia[a] = floorf(o.h);
            ofa[a] = __fadd_rn(__fsub_rn(o.h, oia[a]), o.l);
        }
        oi = f3(oia[0], oia[1], oia[2]);
        of = f3(ofa[0], ofa[1], ofa[2]);
    }
    // the specular cone's direction and aperture first: the view position and normal die here
    float3 rd = f3(0.f, 0.f, 0.f);
    float th = 0.f;
    if (tc.p.specular) {
        float3 vd = norm3(sub3(wp, f3(v.eye[0], v.eye[1], v.eye[2])));
        float dn = dot3(vd, nw);
        rd = norm3(sub3(vd, mul3(nw, __fmul_rn(2.0f, dn))));
        th = fmaxf(rough, tc.p.min_spec_tan_half);
    }
    // Every cone goes through one call site (one inlined copy of the march: the kernel's code stays small in the
    // instruction cache): k < nd the diffuse cones (the normal, then four tilted 60 degrees at phi = 0, 90, 180,
    // 270 degrees), k = nd the specular cone (no precomputed schedule: ns = 0).
    const uint32_t nd = tc.p.diffuse_cones >= 5 ? 5u : 1u;
    const uint32_t ncones = nd + (tc.p.specular ? 1u : 0u);
    // Carried between cones: the origin, the normal, the specular cone and the diffuse sum; the normal's frame
    // is formed again for each diffuse cone (the same operations, so the same directions) rather than kept.
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
    for (uint32_t k = 0; k < ncones; ++k) {
        float3 bx, by, bz;
        coord_space(nw, bx, by, bz);
        float3 dir = bz;
        float tan_half = tc.p.diffuse_tan_half;
        uint32_t ns = kDiffuseSched;
        if (k >= nd) {
            dir = rd, tan_half = th, ns = 0u;
        } else if (k > 0) {
            // bx cos(phi) + by sin(phi) for phi = (k - 1) * 90 degrees (the products by 0 and +-1 are exact)
            const uint32_t j = k - 1;
            float3 side = (j & 1) ? by : bx;
            if (j & 2) side = f3(-side.x, -side.y, -side.z);
            dir = norm3(add3(mul3(bz, tc.cos_tilt), mul3(side, tc.sin_tilt)));
        }
        const float4 c = cone<FMT, ANISO, COUNT>(g, lut, tc, oi, of, dir, tan_half, sched, ns, cnt);
        if (k >= nd) {
            store_out(v.out, v.out_format, npix + pi, c);  // the specular cone is the last
        } else if (nd == 1) {
            acc = c;
        } else if (k == 0) {
            acc = make_float4(__fmul_rn(0.25f, c.x), __fmul_rn(0.25f, c.y), __fmul_rn(0.25f, c.z), __fmul_rn(0.25f, c.w));
        } else {
            acc.x = __fadd_rn(acc.x, __fmul_rn(0.1875f, c.x));
            acc.y = __fadd_rn(acc.y, __fmul_rn(0.1875f, c.y));
            acc.z = __fadd_rn(acc.z, __fmul_rn(0.1875f, c.z));
            acc.w = __fadd_rn(acc.w, __fmul_rn(0.1875f, c.w));
        }
    }
    store_out(v.out, v.out_format, pi, acc);
    if (!tc.p.specular) store_out(v.out, v.out_format, npix + pi, make_float4(0.f, 0.f, 0.f, 0.f));
}

// Work is handed out per warp: a warp tile is TW x (32 / TW) pixels, one lane each, and the warp tiles of all
// views are numbered in view order (tile_base = per-view prefix).  In the one-shot launch (work == nullptr) warp
// w of CTA b traces warp tile b * (TW * TH / 32) + w; in the persistent launch each warp takes tiles from a device
// work counter until the batch is drained (one resident wave of CTAs, so views of different size balance).  A
// warp never waits for the other warps of its CTA: the only CTA barrier is the staging of the tables at the
// start.  The CTA shape and the CTAs resident per SM (MINB) are the variants the tuner picks from.
template <int FMT, bool ANISO, int TW, int TH, int MINB, bool COUNT = false>
__global__ void __launch_bounds__(TW * TH, MINB) trace_kernel(const __grid_constant__ TraceConsts tc,
                                                             const TraceView* __restrict__ views,
                                                             const uint32_t* __restrict__ tile_base, uint32_t nviews,
                                                             uint32_t* work) {
    constexpr int kWarps = TW * TH / 32, WW = TW, WH = 32 / TW;
    static_assert(TW * TH % 32 == 0 && 32 % TW == 0, "warp tiles of 32 pixels");
    uint32_t cnt[2] = {0u, 0u};  // COUNT only: this thread's steps and level samples
    // The diffuse schedule is read from the parameter bank (`tc` is a grid constant): the step index is the same
    // across the warp, so the constant cache broadcasts it without a load-pipe wavefront.
    __shared__ GridRef gs[kWarps];  // the grid of each warp's current view
    __shared__ uint32_t s_lut[3 * kLut];
    for (uint32_t i = threadIdx.x; i < 3 * kLut; i += TW * TH) s_lut[i] = part1by2(i % kLut) << (9 + i / kLut);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    GridRef& g = gs[wid];
    const uint32_t ntiles = tile_base[nviews];
    uint32_t cur_view = 0xffffffffu;
    for (uint32_t it = 0;; ++it) {
        uint32_t tile = 0, vi = 0;
        if (lane == 0) {
            tile = work ? atomicAdd(work, 1u) : (it == 0 ? blockIdx.x * kWarps + wid : ntiles);
            uint32_t lo = 0, hi = nviews;  // last view with tile_base[v] <= tile
            while (hi - lo > 1) {
                uint32_t mid = (lo + hi) / 2;
                if (tile_base[mid] <= tile) lo = mid; else hi = mid;
            }
            vi = lo;
        }
        tile = __shfl_sync(0xffffffffu, tile, 0);
        vi = __shfl_sync(0xffffffffu, vi, 0);
        if (tile >= ntiles) return;
        const TraceView& v = views[vi];
        if (vi != cur_view) {  // stage the view's grid description
            if (lane < kMaxLevels) {
                g.off[lane] = uint32_t(v.off[lane]);
                g.vol[lane] = uint32_t(v.vol[lane]);
            }
            if (lane == 0) {
                g.base = v.grid_base;
                g.dim = v.grid_dim;
                g.levels = v.grid_levels;
                g.tmax = v.tmax;
                // world -> L0 voxel units: (p - origin) * (inv_voxel_fixed / 256) as FP32 pairs, written beside
                // the frame when it was computed
                const FramePairs* fp = reinterpret_cast<const FramePairs*>(v.frame + 1);
                for (int a = 0; a < 3; ++a) g.org_h[a] = fp->org_h[a], g.org_l[a] = fp->org_l[a];
                g.ivs_h = fp->ivs_h;
                g.ivs_l = fp->ivs_l;
            }
            cur_view = vi;
            __syncwarp();
        }
        const uint32_t local = tile - tile_base[vi];
        const uint32_t tiles_x = (v.width + WW - 1) / WW;
        const uint32_t px = (local % tiles_x) * WW + (lane % WW);
        const uint32_t py = (local / tiles_x) * WH + (lane / WW);
        if (px < v.width && py < v.height) trace_pixel<FMT, ANISO, COUNT>(g, s_lut, tc, v, px, py, tc.sched, cnt);
        if constexpr (COUNT) {  // warp totals, one atomic per warp and counter
            const unsigned long long a = __reduce_add_sync(0xffffffffu, cnt[0]), b = __reduce_add_sync(0xffffffffu, cnt[1]);
            if (lane == 0u) {
                atomicAdd(&tc.counts[0], a);
                atomicAdd(&tc.counts[1], b);
            }
            cnt[0] = cnt[1] = 0u;
        }
        __syncwarp();  // g may be restaged for the next tile
    }
}

// Kernel of a variant (host stub address, for cudaLaunchKernel and graph kernel nodes).
template <int FMT, bool ANISO, int V>
const void* variant_fn() {
    constexpr TraceVariant tv = kTraceVariants[V];
    return reinterpret_cast<const void*>(&trace_kernel<FMT, ANISO, int(tv.tw), int(tv.th), int(tv.minb)>);
}

// The instrumented kernel (same outputs, plus the step and sample totals) in the default variant's shape.
template <int FMT, bool ANISO>
const void* count_kernel() {
    constexpr TraceVariant tv = kTraceVariants[trace_default_variant(FMT, ANISO)];
    return reinterpret_cast<const void*>(&trace_kernel<FMT, ANISO, int(tv.tw), int(tv.th), int(tv.minb), true>);
}

template <int FMT, bool ANISO>
const void* kernel_for(uint32_t variant) {
    static_assert(kTraceVariantCount == 5, "one case per variant");
    switch (variant) {
        case 0: return variant_fn<FMT, ANISO, 0>();
        case 1: return variant_fn<FMT, ANISO, 1>();
        case 2: return variant_fn<FMT, ANISO, 2>();
        case 3: return variant_fn<FMT, ANISO, 3>();
        case 4: return variant_fn<FMT, ANISO, 4>();
        default: return nullptr;
    }
}

}  // namespace
}  // namespace f184
