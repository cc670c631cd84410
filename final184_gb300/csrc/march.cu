// march.cu -- the reference-faithful pair: the reference's voxel volume and its single-ray march.
//
// Volume (main.lua:83-144 VoxelGS, :242-275 VoxelPS): every triangle is rasterized at the grid resolution along
// the dominant axis of its face normal (pixel-centre coverage, not conservative); each covered pixel names one
// voxel through the shader's swizzles, including its mixed scales (depth * (dim - 1) against pixel coordinates)
// and its half-pixel offsets; the voxel stores RGB565 albedo in the low 16 bits and the 5-6-5 packed normal in
// the high 16 bits.  The reference keeps the last fragment written (an order that is not defined on a GPU);
// here the highest triangle index wins, which is "last in submission order" made deterministic.
//
// March (indirect.frag:104-222, without the temporal blend): per pixel four rays with a second bounce; a ray
// starts on the surface, takes fixed 0.2-unit steps, loads the voxel each time it enters a new one, and on the
// first non-empty voxel adds the sun's Lambert term behind the shadow-map test (indirect.frag:160-169); a ray that
// takes all its steps without leaving the grid adds the sky term (indirect.frag:178-181).  The reference's sin
// hashes of screen position and frame number (math.inc:83-219) are replaced by an integer hash of (pixel, frame,
// ray), and sin/cos of the sample angle by a Taylor evaluation on an octant: with every FP32 operation written
// with explicit rounding (no contraction), a CPU restatement of the same operation sequence gives the same bits.
#include "gi_device.cuh"

namespace f184 {
namespace {

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return v3(fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x)));
}
__device__ __forceinline__ V3 normalize3(V3 v) {  // v / length(v); a zero vector stays zero
    const float l = __fsqrt_rn(dot3(v, v));
    return l > 0.0f ? v3(fdv(v.x, l), fdv(v.y, l), fdv(v.z, l)) : v;
}

// FP32 maps of the grid frame, rounded from its FP64 fields: world -> voxel coordinates (the reference's
// VoxelProj * VoxelView with the xy * 0.5 + 0.5 and * 128 of indirect.frag:141-143) and world -> shadow clip.
struct MarchMaps {
    float w2v_s, w2v_b[3];
    float w2l[12];
};
__device__ void make_maps(const f184gi_grid_frame* fr, MarchMaps& m) {
    const double inv = fr->inv_voxel_fixed * (1.0 / 256.0);  // exact: a power-of-two scale
    m.w2v_s = __double2float_rn(inv);
    for (int a = 0; a < 3; ++a) m.w2v_b[a] = __double2float_rn(__dmul_rn(-fr->origin[a], inv));
    for (int k = 0; k < 12; ++k) m.w2l[k] = __double2float_rn(fr->light_clip[k]);
}
__device__ __forceinline__ V3 w2v(const MarchMaps& m, V3 p) {
    return v3(fa(fm(p.x, m.w2v_s), m.w2v_b[0]), fa(fm(p.y, m.w2v_s), m.w2v_b[1]), fa(fm(p.z, m.w2v_s), m.w2v_b[2]));
}
__device__ __forceinline__ float w2l_row(const float* r, V3 p) {
    return fa(fa(fa(fm(r[0], p.x), fm(r[1], p.y)), fm(r[2], p.z)), r[3]);
}

// ---------------- reference volume ----------------

struct RefTri {
    int32_t X[3], Y[3];  // screen position, 24.8 fixed point pixels, counter-clockwise
    float z0, a, b;      // depth at the centre (X, Y): (z0 + a (X - X[0])) + b (Y - Y[0])
    int32_t x0, x1, y0, y1;  // pixel box (inclusive), empty when x0 > x1
    uint32_t orient;
};

// Per triangle: orientation by the dominant axis of the face normal in grid axes (VoxelGS's rule: X if
// |n.x| > |n.y| and |n.x| > |n.z|, Y if |n.y| > |n.x| and |n.y| > |n.z|, else Z), the swizzled screen position
// in pixels (x, y) and depth in [0, 1]:  Z: (u.x, u.y, u.z / dim);  X: (u.z, u.y, 1 - u.x / dim);
// Y: (u.x, dim - u.z, u.y / dim), snapped to 1/256 pixel; the depth plane solved in FP64, kept in FP32.
__global__ void __launch_bounds__(128) refvox_setup(const float* __restrict__ tri, uint64_t ntris,
                                                   const f184gi_grid_frame* __restrict__ fr, uint32_t dim,
                                                   RefTri* __restrict__ recs, uint32_t* status) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    MarchMaps m;
    make_maps(fr, m);
    V3 u[3];
    for (int v = 0; v < 3; ++v) {
        const float* p = tri + t * 9 + 3 * v;
        u[v] = w2v(m, v3(p[0], p[1], p[2]));
    }
    RefTri r;
    r.x0 = 1, r.x1 = 0, r.y0 = 1, r.y1 = 0;
    const V3 n = cross3(v3(fs(u[1].x, u[0].x), fs(u[1].y, u[0].y), fs(u[1].z, u[0].z)),
                        v3(fs(u[2].x, u[0].x), fs(u[2].y, u[0].y), fs(u[2].z, u[0].z)));
    const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
    const uint32_t o = ax > ay ? (ax > az ? 1u : 0u) : (ay > az ? 2u : 0u);
    r.orient = o;
    const float fd = float(dim), inv_dim = 1.0f / fd;  // exact: dim is a power of two
    float sx[3], sy[3], sz[3];
    for (int v = 0; v < 3; ++v) {
        if (o == 0) sx[v] = u[v].x, sy[v] = u[v].y, sz[v] = fm(u[v].z, inv_dim);
        else if (o == 1) sx[v] = u[v].z, sy[v] = u[v].y, sz[v] = fs(1.0f, fm(u[v].x, inv_dim));
        else sx[v] = u[v].x, sy[v] = fs(fd, u[v].z), sz[v] = fm(u[v].y, inv_dim);
        if (!(fabsf(sx[v]) < 4096.0f && fabsf(sy[v]) < 4096.0f)) {  // far outside the grid (or not finite)
            set_status(status, kStatusRange);
            recs[t] = r;
            return;
        }
    }
    int32_t X[3], Y[3];
    for (int v = 0; v < 3; ++v) X[v] = __float2int_rn(fm(sx[v], 256.0f)), Y[v] = __float2int_rn(fm(sy[v], 256.0f));
    int64_t det = int64_t(X[1] - X[0]) * (Y[2] - Y[0]) - int64_t(X[2] - X[0]) * (Y[1] - Y[0]);
    if (det == 0) {
        recs[t] = r;
        return;
    }
    int i1 = 1, i2 = 2;
    if (det < 0) i1 = 2, i2 = 1, det = -det;
    const int id[3] = {0, i1, i2};
    for (int v = 0; v < 3; ++v) r.X[v] = X[id[v]], r.Y[v] = Y[id[v]];
    const double z0 = sz[0], z1 = sz[i1], z2 = sz[i2];
    const double dx1 = double(r.X[1] - r.X[0]), dy1 = double(r.Y[1] - r.Y[0]);
    const double dx2 = double(r.X[2] - r.X[0]), dy2 = double(r.Y[2] - r.Y[0]);
    const double dz1 = __dsub_rn(z1, z0), dz2 = __dsub_rn(z2, z0);
    const double dd = double(det);
    r.z0 = float(z0);
    r.a = __double2float_rn(__ddiv_rn(__dsub_rn(__dmul_rn(dz1, dy2), __dmul_rn(dz2, dy1)), dd));
    r.b = __double2float_rn(__ddiv_rn(__dsub_rn(__dmul_rn(dz2, dx1), __dmul_rn(dz1, dx2)), dd));
    int32_t mnx = min(r.X[0], min(r.X[1], r.X[2])), mxx = max(r.X[0], max(r.X[1], r.X[2]));
    int32_t mny = min(r.Y[0], min(r.Y[1], r.Y[2])), mxy = max(r.Y[0], max(r.Y[1], r.Y[2]));
    // pixel centres (256 p + 128) inside [mn, mx]
    r.x0 = max(0, (mnx - 128 + 255) >> 8), r.x1 = min(int32_t(dim) - 1, (mxx - 128) >> 8);
    r.y0 = max(0, (mny - 128 + 255) >> 8), r.y1 = min(int32_t(dim) - 1, (mxy - 128) >> 8);
    recs[t] = r;
}

// One warp per triangle: every pixel of its box; a centre on an edge belongs to the triangle when the edge runs
// down the screen (dy > 0) or, horizontal, leftwards (dy == 0, dx < 0): of two triangles sharing an edge exactly
// one takes it.  The covered voxel records the highest triangle index + 1.
__global__ void __launch_bounds__(256) refvox_raster(const RefTri* __restrict__ recs, uint64_t ntris, uint32_t dim,
                                                    uint32_t* __restrict__ owner) {
    const uint64_t t = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (t >= ntris) return;
    const RefTri r = recs[t];
    if (r.x0 > r.x1 || r.y0 > r.y1) return;
    const uint32_t bw = uint32_t(r.x1 - r.x0 + 1), bh = uint32_t(r.y1 - r.y0 + 1);
    const float maxd = float(dim - 1);
    int64_t ex[3], ey[3];
    bool incl[3];
    for (int e = 0; e < 3; ++e) {
        const int n = (e + 1) % 3;
        ex[e] = int64_t(r.X[n]) - r.X[e];
        ey[e] = int64_t(r.Y[n]) - r.Y[e];
        incl[e] = ey[e] > 0 || (ey[e] == 0 && ex[e] < 0);
    }
    for (uint32_t k = lane; k < bw * bh; k += 32) {
        const int32_t px = r.x0 + int32_t(k % bw), py = r.y0 + int32_t(k / bw);
        const int64_t cx = int64_t(px) * 256 + 128, cy = int64_t(py) * 256 + 128;
        bool in = true;
        for (int e = 0; e < 3; ++e) {
            const int64_t w = ex[e] * (cy - r.Y[e]) - ey[e] * (cx - r.X[e]);
            in = in && (w > 0 || (w == 0 && incl[e]));
        }
        if (!in) continue;
        const float z = fa(fa(r.z0, fm(r.a, float(cx - r.X[0]))), fm(r.b, float(cy - r.Y[0])));
        int vx, vy, vz;
        if (r.orient == 0) {
            vx = px, vy = py, vz = __float2int_rz(fm(z, maxd));
        } else if (r.orient == 1) {
            vx = __float2int_rz(fm(fs(1.0f, z), maxd)), vy = py, vz = px;
        } else {
            vx = px, vy = __float2int_rz(fm(z, maxd)), vz = __float2int_rz(fs(maxd, fa(float(py), 0.5f)));
        }
        if (unsigned(vx) >= dim || unsigned(vy) >= dim || unsigned(vz) >= dim) continue;
        atomicMax(&owner[(uint64_t(vz) * dim + uint64_t(vy)) * dim + uint64_t(vx)], uint32_t(t + 1));
    }
}

// Voxel = RGB565 albedo | 565 normal << 16 of its owner (VoxelPS's packing; the normal is the owner's face
// normal in world space, each packed field clamped at 0 where n * 16 + 15 would be negative).
__global__ void __launch_bounds__(256) refvox_resolve(const uint32_t* __restrict__ owner, uint64_t nvox,
                                                     const float* __restrict__ tri,
                                                     const uint32_t* __restrict__ albedo,
                                                     uint32_t* __restrict__ vol) {
    const uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= nvox) return;
    const uint32_t o = owner[v];
    if (!o) {
        vol[v] = 0;
        return;
    }
    const uint64_t t = o - 1;
    const uint32_t al = albedo[t];
    const float cr = fdv(float(al & 255u), 255.0f), cg = fdv(float((al >> 8) & 255u), 255.0f),
                cb = fdv(float((al >> 16) & 255u), 255.0f);
    const uint32_t color = (__float2uint_rz(fm(cr, 31.0f)) << 11) | (__float2uint_rz(fm(cg, 63.0f)) << 5) |
                           __float2uint_rz(fm(cb, 31.0f));
    const float* p = tri + t * 9;
    const V3 n = normalize3(cross3(v3(fs(p[3], p[0]), fs(p[4], p[1]), fs(p[5], p[2])),
                                   v3(fs(p[6], p[0]), fs(p[7], p[1]), fs(p[8], p[2]))));
    const uint32_t nx = __float2uint_rz(fmaxf(0.0f, fa(fm(n.x, 16.0f), 15.0f)));
    const uint32_t ny = __float2uint_rz(fmaxf(0.0f, fa(fm(n.y, 32.0f), 31.0f)));
    const uint32_t nz = __float2uint_rz(fmaxf(0.0f, fa(fm(n.z, 16.0f), 15.0f)));
    const uint32_t normal = ((nx << 11) | (ny << 5) | nz) & 0xffffu;
    vol[v] = (color & 0xffffu) | (normal << 16);
}

// ---------------- march ----------------

// lowbias32 (C. Wellons' integer hash): the per-pixel random numbers, 24 bits each.
__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// sin and cos of 2 pi v for v in [0, 1): the quadrant from v, the remainder r in [-1/8, 1/8] turn (exact), then
// the Taylor series of sin (to x^9) and cos (to x^10) at x = 2 pi r, |x| <= pi/4 (truncation < 2e-9).
__device__ __forceinline__ void sincos_turns(float v, float& s, float& c) {
    const int q = __float2int_rd(fa(fm(v, 4.0f), 0.5f));
    const float r = fs(v, fm(float(q), 0.25f));
    const float x = fm(r, 6.28318530717958647692f);
    const float x2 = fm(x, x);
    float ps = fa(-1.0f / 5040.0f, fm(x2, 1.0f / 362880.0f));
    ps = fa(1.0f / 120.0f, fm(x2, ps));
    ps = fa(-1.0f / 6.0f, fm(x2, ps));
    ps = fa(1.0f, fm(x2, ps));
    const float sn = fm(x, ps);
    float pc = fa(1.0f / 40320.0f, fm(x2, -1.0f / 3628800.0f));
    pc = fa(-1.0f / 720.0f, fm(x2, pc));
    pc = fa(1.0f / 24.0f, fm(x2, pc));
    pc = fa(-0.5f, fm(x2, pc));
    const float cs = fa(1.0f, fm(x2, pc));
    switch (q & 3) {
        case 0: s = sn, c = cs; break;
        case 1: s = cs, c = -sn; break;
        case 2: s = -sn, c = -cs; break;
        default: s = -cs, c = sn; break;
    }
}

// make_coord_space (indirect.frag:71-86): the columns x, y, z of the ray frame.
__device__ __forceinline__ void coord_space(V3 n, V3& x, V3& y, V3& z) {
    V3 h = n;
    const float ax = fabsf(h.x), ay = fabsf(h.y), az = fabsf(h.z);
    if (ax <= ay && ax <= az) h.x = 1.0f;
    else if (ay <= ax && ay <= az) h.y = 1.0f;
    else h.z = 1.0f;
    z = normalize3(n);
    y = normalize3(cross3(h, z));
    x = normalize3(cross3(z, y));
}

__device__ __forceinline__ float smoothstep01(float e1, float x) {  // smoothstep(0, e1, x)
    float t = fdv(x, e1);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return fm(fm(t, t), fs(3.0f, fm(2.0f, t)));
}

struct Hit {
    V3 wpos, wnorm, brdf;
    bool hit;
};

struct MarchShared {
    MarchMaps maps;
    float pow5[32], pow6[64];
};

// getIndirect (indirect.frag:104-184) for one ray; `seed` is the reference's randSeed (0..7).
__device__ V3 march_ray(const MarchShared& sh, const MarchJobDev& J, uint32_t pix, V3 wpos, V3 wnorm, uint32_t seed,
                        Hit& hit) {
    hit.hit = false;
    V3 lo = v3(0.0f, 0.0f, 0.0f);
    const uint32_t key = lowbias32(J.p.frame * 16u + seed * 2u);
    const float ru = fm(float(lowbias32(pix ^ key) >> 8), 5.9604644775390625e-8f);
    const float rv = fm(float(lowbias32(pix ^ (key + 0x9e3779b9u)) >> 8), 5.9604644775390625e-8f);
    // hemisphereSample_cos (math.inc:76-81)
    const float ct = __fsqrt_rn(fs(1.0f, ru));
    const float st = __fsqrt_rn(fs(1.0f, fm(ct, ct)));
    float sp, cp;
    sincos_turns(rv, sp, cp);
    const V3 dl = v3(fm(cp, st), fm(sp, st), ct);
    V3 bx, by, bz;
    coord_space(wnorm, bx, by, bz);
    V3 dir = v3(fa(fa(fm(bx.x, dl.x), fm(by.x, dl.y)), fm(bz.x, dl.z)),
                fa(fa(fm(bx.y, dl.x), fm(by.y, dl.y)), fm(bz.y, dl.z)),
                fa(fa(fm(bx.z, dl.x), fm(by.z, dl.y)), fm(bz.z, dl.z)));
    if (dot3(dir, wnorm) < 0.0f) dir = v3(-dir.x, -dir.y, -dir.z);
    const float ndd = dot3(dir, wnorm);
    const float step = J.p.step_size;
    const float so = fa(1.0f, rv);
    V3 mp = v3(fa(wpos.x, fdv(fm(fm(dir.x, so), step), ndd)), fa(wpos.y, fdv(fm(fm(dir.y, so), step), ndd)),
               fa(wpos.z, fdv(fm(fm(dir.z, so), step), ndd)));
    const V3 sv = w2v(sh.maps, wpos);
    int px = __float2int_rz(sv.x), py = __float2int_rz(sv.y), pz = __float2int_rz(sv.z);
    const float maxd = float(J.dim - 1);
    uint32_t i = 0;
    for (; i < J.p.max_steps; ++i) {
        mp = v3(fa(mp.x, fm(dir.x, step)), fa(mp.y, fm(dir.y, step)), fa(mp.z, fm(dir.z, step)));
        const V3 vp = w2v(sh.maps, mp);
        if (vp.x < 0.0f || vp.y < 0.0f || vp.z < 0.0f || vp.x > maxd || vp.y > maxd || vp.z > maxd) break;
        const int ix = __float2int_rz(vp.x), iy = __float2int_rz(vp.y), iz = __float2int_rz(vp.z);
        if (ix == px && iy == py && iz == pz) continue;
        const uint32_t data = J.vol[(uint64_t(iz) * J.dim + uint64_t(iy)) * J.dim + uint64_t(ix)];
        px = ix, py = iy, pz = iz;
        const uint32_t r = data & 0xffffu, g = data >> 16;
        if (r == 0) continue;
        const V3 col = v3(sh.pow5[(r >> 11) & 31u], sh.pow6[(r >> 5) & 63u], sh.pow5[r & 31u]);
        const V3 vn = normalize3(v3(fs(fdv(float(g & 0x1fu), 16.0f), 1.0f),
                                    fs(fdv(float((g >> 5) & 0x3fu), 32.0f), 1.0f),
                                    fs(fdv(float((g >> 11) & 0x1fu), 16.0f), 1.0f)));
        // first-bounce lighting: shadow map at the voxel position pushed along its normal
        const V3 q = v3(fa(mp.x, fm(vn.x, J.p.normal_offset)), fa(mp.y, fm(vn.y, J.p.normal_offset)),
                        fa(mp.z, fm(vn.z, J.p.normal_offset)));
        const float lx = w2l_row(sh.maps.w2l, q), ly = w2l_row(sh.maps.w2l + 4, q), lz = w2l_row(sh.maps.w2l + 8, q);
        const int tx = __float2int_rz(fm(fa(fm(lx, 0.5f), 0.5f), float(J.res)));
        const int ty = __float2int_rz(fm(fa(fm(ly, 0.5f), 0.5f), float(J.res)));
        float shade = 1.0f;  // outside the map: lit
        if (unsigned(tx) < J.res && unsigned(ty) < J.res) {
            const unsigned long long k = J.shadow[uint64_t(ty) * J.res + uint64_t(tx)];
            const float sd = k == ~0ull ? 1.0f : __uint_as_float(uint32_t(k >> 32));
            shade = sd < fa(lz, J.p.shadow_bias) ? 0.0f : 1.0f;
        }
        const float lam = fabsf(dot3(v3(-J.light_dir[0], -J.light_dir[1], -J.light_dir[2]), vn));
        const float den = fmaxf(0.01f, ndd);
        const V3 br = v3(fdv(fm(lam, col.x), den), fdv(fm(lam, col.y), den), fdv(fm(lam, col.z), den));
        hit.brdf = br;
        lo = v3(fa(lo.x, fm(fm(J.lum[0], shade), br.x)), fa(lo.y, fm(fm(J.lum[1], shade), br.y)),
                fa(lo.z, fm(fm(J.lum[2], shade), br.z)));
        hit.wpos = mp;
        hit.wnorm = vn;
        hit.hit = true;
        break;
    }
    if (!hit.hit && i == J.p.max_steps) {
        const float den = fmaxf(0.01f, ndd);
        const float ss = smoothstep01(0.01f, ndd);
        lo = v3(fa(lo.x, fm(fdv(fm(J.p.sky[0], J.p.sky_scale), den), ss)),
                fa(lo.y, fm(fdv(fm(J.p.sky[1], J.p.sky_scale), den), ss)),
                fa(lo.z, fm(fdv(fm(J.p.sky[2], J.p.sky_scale), den), ss)));
    }
    return lo;
}

// Eight CTAs of 256 threads per SM (32 registers, a few bytes spilled): each step of a ray is a dependent gather
// from the volume, so the march wants warps to hide it (per 1080p view: 2.70 ms at 3 CTAs per SM and 68
// registers, 2.32 / 2.08 / 1.98 at 4 / 5 / 6, 1.84 at 7 or 8).  Its arithmetic is written out operation by
// operation, so the bits do not depend on the register budget.
__global__ void __launch_bounds__(256, 8) march_kernel(MarchJobDev J, MarchViewDev v) {
    __shared__ MarchShared sh;
    if (threadIdx.x == 0 && threadIdx.y == 0) make_maps(J.frame_ptr, sh.maps);
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (uint32_t k = tid; k < 96; k += blockDim.x * blockDim.y) {
        if (k < 32) sh.pow5[k] = J.pow5[k];
        else sh.pow6[k - 32] = J.pow6[k - 32];
    }
    __syncthreads();
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= v.width || py >= v.height) return;
    const uint64_t pi = uint64_t(py) * v.width + px;
    const float d = v.depth[pi];
    float4* out = static_cast<float4*>(v.out);
    if (!(d < 1.0f)) {
        out[pi] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    // G-buffer decode (indirect.frag:44-58, 189-196): the projective rows in FP64, as in the cone trace
    const float nx = fs(fm(fdv(fa(float(px), 0.5f), float(v.width)), 2.0f), 1.0f);
    const float ny = fs(fm(fdv(fa(float(py), 0.5f), float(v.height)), 2.0f), 1.0f);
    const float* ip = v.iproj;
    const float vx = fa(fa(fa(fm(ip[0], nx), fm(ip[1], ny)), fm(ip[2], d)), ip[3]);
    const float vy = fa(fa(fa(fm(ip[4], nx), fm(ip[5], ny)), fm(ip[6], d)), ip[7]);
    const double* iz = v.iproj_zw;
    const double dnx = nx, dny = ny, dd = d;
    const double vz = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(iz[0], dnx), __dmul_rn(iz[1], dny)), __dmul_rn(iz[2], dd)), iz[3]);
    const double vw = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(iz[4], dnx), __dmul_rn(iz[5], dny)), __dmul_rn(iz[6], dd)), iz[7]);
    const double rw = __ddiv_rn(1.0, vw);
    const float rwf = __double2float_rn(rw);
    const V3 cs = v3(fm(vx, rwf), fm(vy, rwf), __double2float_rn(__dmul_rn(vz, rw)));
    const float* iv = v.iview;
    const V3 wpos = v3(fa(fa(fa(fm(iv[0], cs.x), fm(iv[1], cs.y)), fm(iv[2], cs.z)), iv[3]),
                       fa(fa(fa(fm(iv[4], cs.x), fm(iv[5], cs.y)), fm(iv[6], cs.z)), iv[7]),
                       fa(fa(fa(fm(iv[8], cs.x), fm(iv[9], cs.y)), fm(iv[10], cs.z)), iv[11]));
    // view-space normal (octahedral FP16 pair), then mat3(InvModelView) without renormalising (indirect.frag:200)
    const uint32_t pn = v.normal[pi];
    V3 on = v3(__half2float(__ushort_as_half(uint16_t(pn & 0xffffu))),
               __half2float(__ushort_as_half(uint16_t(pn >> 16))), 0.0f);
    on.z = fs(fs(1.0f, fabsf(on.x)), fabsf(on.y));
    if (on.z < 0.0f) {
        const float ox = on.x, oy = on.y;
        on.x = fm(fs(1.0f, fabsf(oy)), ox >= 0.0f ? 1.0f : -1.0f);
        on.y = fm(fs(1.0f, fabsf(ox)), oy >= 0.0f ? 1.0f : -1.0f);
    }
    const V3 cn = normalize3(on);
    const V3 wn = v3(fa(fa(fm(iv[0], cn.x), fm(iv[1], cn.y)), fm(iv[2], cn.z)),
                     fa(fa(fm(iv[4], cn.x), fm(iv[5], cn.y)), fm(iv[6], cn.z)),
                     fa(fa(fm(iv[8], cn.x), fm(iv[9], cn.y)), fm(iv[10], cn.z)));
    const uint32_t pix = uint32_t(pi);
    V3 acc = v3(0.0f, 0.0f, 0.0f);
    Hit h;
    for (uint32_t k = 0; k < J.p.rays; ++k) {
        const V3 l1 = march_ray(sh, J, pix, wpos, wn, 2 * k, h);
        acc = v3(fa(acc.x, l1.x), fa(acc.y, l1.y), fa(acc.z, l1.z));
        if (h.hit && J.p.second_bounce) {
            const V3 br = h.brdf;
            Hit h2;
            const V3 l2 = march_ray(sh, J, pix, h.wpos, h.wnorm, 2 * k + 1, h2);
            acc = v3(fa(acc.x, fm(br.x, l2.x)), fa(acc.y, fm(br.y, l2.y)), fa(acc.z, fm(br.z, l2.z)));
        }
    }
    const float sc = fdv(1.0f, float(J.p.rays));
    out[pi] = make_float4(fm(acc.x, sc), fm(acc.y, sc), fm(acc.z, sc), -cs.z);
}

}  // namespace

size_t refvox_scratch_bytes(uint64_t ntris, uint32_t dim) {
    return ((ntris * sizeof(RefTri) + 255) / 256) * 256 + uint64_t(dim) * dim * dim * 4 + 256;
}

int refvox_launch(const float* tri, const uint32_t* albedo, uint64_t ntris, const f184gi_grid_frame* d_frame,
                  uint32_t dim, uint32_t* vol, void* scratch, size_t scratch_bytes, uint32_t* d_status,
                  cudaStream_t s) {
    if (scratch_bytes < refvox_scratch_bytes(ntris, dim)) return fail(F184GI_ERR_INVALID, "refvox: scratch too small");
    RefTri* recs = static_cast<RefTri*>(scratch);
    uint32_t* owner = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + ((ntris * sizeof(RefTri) + 255) / 256) * 256);
    const uint64_t nvox = uint64_t(dim) * dim * dim;
    cudaError_t e = cudaMemsetAsync(owner, 0, nvox * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "refvox: clear");
    if (ntris) {
        refvox_setup<<<uint32_t((ntris + 127) / 128), 128, 0, s>>>(tri, ntris, d_frame, dim, recs, d_status);
        refvox_raster<<<uint32_t((ntris * 32 + 255) / 256), 256, 0, s>>>(recs, ntris, dim, owner);
        note_launches(2);
    }
    refvox_resolve<<<uint32_t((nvox + 255) / 256), 256, 0, s>>>(owner, nvox, tri, albedo, vol);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "refvox");
}

int march_launch(const MarchJobDev& job, const MarchViewDev& view, cudaStream_t s) {
    const dim3 block(16, 16);
    const dim3 grid((view.width + 15) / 16, (view.height + 15) / 16);
    march_kernel<<<grid, block, 0, s>>>(job, view);
    note_launches(1);
    return cuda_fail(cudaGetLastError(), "march");
}

}  // namespace f184
