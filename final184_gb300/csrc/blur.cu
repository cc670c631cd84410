// blur.cu -- the depth-aware (cross-bilateral) blur of the indirect image: the reference's two passes
// blurX/blurY over Shader/Lighting/bilateralBlur.inc:19-73 (MegaPipeline.cpp:270-284).
//
// Each pass weighs 1 + 2 * 6 taps along one axis: offsets +-2, 4, 6, 8 pixels with r = 1..4, then +-11 and +-15
// pixels with r = 5 and 7 (the shader's offsets are in units of 2 / resolution and its half-texel steps land on
// texel centres, so the linear sampler reads single texels), clamped at the image edge.  Weight
// exp2(-r^2 / 32 - (512 (z0 - z))^2) with z the G-buffer depth.  The first pass runs along the rows' index (the
// reference's blurX shifts v), the second along x; the output alpha is 0 as in the shader.  exp2 is evaluated
// as 2^n times a degree-7 Taylor polynomial of e^(f ln 2), f = t - round(t), with explicit rounding, so a CPU
// restatement of the same sequence gives the same bits.
#include "gi_device.cuh"

namespace f184 {
namespace {

__device__ __forceinline__ float exp2_poly(float t) {
    if (!(t > -126.0f)) return 0.0f;
    t = fminf(t, 127.0f);
    const int n = __float2int_rn(t);
    const float x = __fmul_rn(__fsub_rn(t, float(n)), 0.693147180559945309f);
    float p = __fadd_rn(1.0f / 720.0f, __fmul_rn(x, 1.0f / 5040.0f));
    p = __fadd_rn(1.0f / 120.0f, __fmul_rn(x, p));
    p = __fadd_rn(1.0f / 24.0f, __fmul_rn(x, p));
    p = __fadd_rn(1.0f / 6.0f, __fmul_rn(x, p));
    p = __fadd_rn(0.5f, __fmul_rn(x, p));
    p = __fadd_rn(1.0f, __fmul_rn(x, p));
    p = __fadd_rn(1.0f, __fmul_rn(x, p));
    return __fmul_rn(p, __int_as_float((n + 127) << 23));
}

__device__ __forceinline__ float cross_weight(float r, float d, float d0) {
    const float dz = __fmul_rn(__fsub_rn(d0, d), 512.0f);
    return exp2_poly(__fsub_rn(__fmul_rn(__fmul_rn(-r, r), 1.0f / 32.0f), __fmul_rn(dz, dz)));
}

__global__ void __launch_bounds__(256) blur_pass(const float4* __restrict__ in, const float* __restrict__ depth,
                                                uint32_t W, uint32_t H, int axis, float4* __restrict__ out) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int n = axis ? int(W) : int(H);
    const int c = axis ? int(x) : int(y);
    auto at = [&](int k) -> uint64_t {  // pixel k along the axis, clamped
        k = k < 0 ? 0 : (k >= n ? n - 1 : k);
        return axis ? uint64_t(y) * W + uint64_t(k) : uint64_t(k) * W + x;
    };
    const uint64_t p0 = uint64_t(y) * W + x;
    const float4 s0 = in[p0];
    const float z0 = depth[p0];
    float tr = s0.x, tg = s0.y, tb = s0.z, tw = 1.0f;
    auto tap = [&](int off, float r) {
        const uint64_t q = at(c + off);
        const float4 s = in[q];
        const float w = cross_weight(r, depth[q], z0);
        tr = __fadd_rn(tr, __fmul_rn(s.x, w));
        tg = __fadd_rn(tg, __fmul_rn(s.y, w));
        tb = __fadd_rn(tb, __fmul_rn(s.z, w));
        tw = __fadd_rn(tw, w);
    };
#pragma unroll
    for (int i = 1; i <= 4; ++i) {
        tap(2 * i, float(i));
        tap(-2 * i, float(i));
    }
#pragma unroll
    for (int i = 5; i <= 7; i += 2) {
        tap(2 * i + 1, float(i));
        tap(-2 * i - 1, float(i));
    }
    out[p0] = make_float4(__fdiv_rn(tr, tw), __fdiv_rn(tg, tw), __fdiv_rn(tb, tw), 0.0f);
}

}  // namespace

int blur_launch(const float* in, const float* depth, uint32_t W, uint32_t H, float* tmp, float* out, cudaStream_t s) {
    const dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    blur_pass<<<grid, block, 0, s>>>(reinterpret_cast<const float4*>(in), depth, W, H, 0,
                                     reinterpret_cast<float4*>(tmp));
    blur_pass<<<grid, block, 0, s>>>(reinterpret_cast<const float4*>(tmp), depth, W, H, 1,
                                     reinterpret_cast<float4*>(out));
    note_launches(2);
    return cuda_fail(cudaGetLastError(), "blur");
}

}  // namespace f184
