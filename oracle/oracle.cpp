// oracle.cpp -- CPU restatement of the voxel GI path.  TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Build with -ffp-contract=off and without -ffast-math: the discrete decisions below rely on every FP64
// operation being rounded on its own, in the order written, so that they agree bit for bit with the device.
//
// Reference lines restated here (paths relative to the reference project):
//   VoxelGS dominant axis          Pipelang/Internal/main.lua:93-115
//   VoxelPS address + 565 packing  Pipelang/Internal/main.lua:242-275
//   565 unpack / make_coord_space  Shader/Lighting/indirect.frag:71-102
//   Lambert + shadow compare       Shader/Lighting/indirect.frag:60-62, 160-169
//   hemisphereSample_cos           Shader/math.inc:76-81
//   G-buffer decode                Shader/Lighting/indirect.frag:44-58, 189-196
//   camera conventions             Foreground/SceneGraph/Camera.cpp:85-111

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

constexpr int64_t kVoxelFixed = 256;   // 24.8 fixed point: units per voxel
constexpr int64_t kHalfVoxel = 128;
constexpr int64_t kMaxFixed = int64_t(1) << 19;
constexpr double kGuard = 16.0;        // raster guard band in NDC units

int nthreads_or_default(int n) {
    if (n > 0) return n;
    unsigned h = std::thread::hardware_concurrency();
    return h ? int(h) : 1;
}

template <class F>
void parallel_for(int64_t begin, int64_t end, int nthreads, F&& fn) {
    int64_t n = end - begin;
    if (n <= 0) return;
    int nt = int(std::min<int64_t>(nthreads_or_default(nthreads), n));
    if (nt <= 1) {
        fn(begin, end);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        int64_t b = begin + n * t / nt, e = begin + n * (t + 1) / nt;
        th.emplace_back([&fn, b, e] { fn(b, e); });
    }
    for (auto& x : th) x.join();
}

inline int64_t floor_div(int64_t a, int64_t b) {  // b > 0
    int64_t q = a / b;
    if ((a % b) != 0 && (a < 0)) --q;
    return q;
}

inline uint32_t float_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float bits_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// row . (x, y, z, 1), each product and sum rounded in this order
inline double mrow(const double* r, double x, double y, double z) {
    double a = r[0] * x;
    double b = r[1] * y;
    double c = r[2] * z;
    double s = a + b;
    s = s + c;
    return s + r[3];
}

struct V4 {
    double x, y, z, w;
};

double plane_dist(int k, const V4& v) {
    switch (k) {
        case 0: return v.z;
        case 1: return v.w - v.z;
        case 2: return kGuard * v.w - v.x;
        case 3: return v.x + kGuard * v.w;
        case 4: return kGuard * v.w - v.y;
        default: return v.y + kGuard * v.w;
    }
}

// Sutherland-Hodgman against the six planes; returns the polygon size (0 when culled).
int clip_polygon(V4* poly, int n) {
    V4 tmp[12];
    for (int k = 0; k < 6; ++k) {
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const V4& a = poly[i];
            const V4& b = poly[(i + 1) % n];
            double da = plane_dist(k, a), db = plane_dist(k, b);
            bool ina = da >= 0.0, inb = db >= 0.0;
            if (ina) tmp[m++] = a;
            if (ina != inb) {
                double t = da / (da - db);
                V4 r;
                r.x = a.x + t * (b.x - a.x);
                r.y = a.y + t * (b.y - a.y);
                r.z = a.z + t * (b.z - a.z);
                r.w = a.w + t * (b.w - a.w);
                tmp[m++] = r;
            }
        }
        n = m;
        if (n < 3) return 0;
        for (int i = 0; i < n; ++i) poly[i] = tmp[i];
    }
    return n;
}

// Float-float arithmetic (unevaluated FP32 pairs), the device's operations one for one (this file is compiled
// without contraction, so each operation rounds once): the rasterizer's plane solve and the trace's pixel set-up.
struct FF32 {
    float h, l;
};
inline void ff_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
inline FF32 ff_norm(float s, float e) {
    const float h = s + e;
    return FF32{h, e - (h - s)};
}
inline FF32 ff_add(FF32 a, FF32 b) {
    float s, e;
    ff_two_sum(a.h, b.h, s, e);
    return ff_norm(s, e + (a.l + b.l));
}
inline FF32 ff_mul(FF32 a, FF32 b) {
    const float p = a.h * b.h;
    const float e = std::fma(a.h, b.l, std::fma(a.l, b.h, std::fma(a.h, b.h, -p)));
    return ff_norm(p, e);
}
inline FF32 ff_div(FF32 a, FF32 b) {
    const float q = a.h / b.h;
    const FF32 r = ff_add(a, ff_mul(FF32{-q, 0.0f}, b));
    return ff_norm(q, r.h / b.h);
}

// Snapped triangle: vertices in 1/16 pixel, depth plane z(X, Y) = z0 + a (X - X0) + b (Y - Y0) with
// z0, a, b rounded to FP32 from a float-float plane solve (FP32 depths) or an FP64 one (a clipped triangle).
struct SnapTri {
    int64_t X[3], Y[3];
    double Z[3];
    bool f32z = false;  // Z holds FP32 values (a triangle inside the clip volume)
    int64_t area2;
    float z0, a, b;
    int64_t x0, x1, y0, y1;  // pixel range, inclusive
};

// orientation, depth plane (rounded to FP32) and pixel range of a triangle already snapped to X, Y, Z
// (raster.cu snap_finish)
bool snap_finish(SnapTri& s, uint32_t W, uint32_t H) {
    int64_t area2 = (s.X[1] - s.X[0]) * (s.Y[2] - s.Y[0]) - (s.Y[1] - s.Y[0]) * (s.X[2] - s.X[0]);
    if (area2 == 0) return false;
    if (area2 < 0) {
        std::swap(s.X[1], s.X[2]);
        std::swap(s.Y[1], s.Y[2]);
        std::swap(s.Z[1], s.Z[2]);
        area2 = -area2;
    }
    s.area2 = area2;
    if (s.f32z) {
        const float z0 = float(s.Z[0]), z1 = float(s.Z[1]), z2 = float(s.Z[2]);
        FF32 dz1, dz2;
        ff_two_sum(z1, -z0, dz1.h, dz1.l);
        ff_two_sum(z2, -z0, dz2.h, dz2.l);
        const float dx1 = float(s.X[1] - s.X[0]), dy1 = float(s.Y[1] - s.Y[0]);
        const float dx2 = float(s.X[2] - s.X[0]), dy2 = float(s.Y[2] - s.Y[0]);
        const float dh = float(area2);
        const FF32 D{dh, float(area2 - int64_t(dh))};
        const FF32 na = ff_add(ff_mul(dz1, FF32{dy2, 0.0f}), ff_mul(dz2, FF32{-dy1, 0.0f}));
        const FF32 nb = ff_add(ff_mul(dz2, FF32{dx1, 0.0f}), ff_mul(dz1, FF32{-dx2, 0.0f}));
        s.z0 = z0;
        s.a = ff_div(na, D).h;
        s.b = ff_div(nb, D).h;
    } else {
        double dx1 = double(s.X[1] - s.X[0]), dy1 = double(s.Y[1] - s.Y[0]);
        double dx2 = double(s.X[2] - s.X[0]), dy2 = double(s.Y[2] - s.Y[0]);
        double dz1 = s.Z[1] - s.Z[0], dz2 = s.Z[2] - s.Z[0];
        double D = double(area2);
        double na = dz1 * dy2;
        na = na - dz2 * dy1;
        double nb = dz2 * dx1;
        nb = nb - dz1 * dx2;
        s.z0 = float(s.Z[0]);
        s.a = float(na / D);
        s.b = float(nb / D);
    }
    int64_t mnx = std::min({s.X[0], s.X[1], s.X[2]}), mxx = std::max({s.X[0], s.X[1], s.X[2]});
    int64_t mny = std::min({s.Y[0], s.Y[1], s.Y[2]}), mxy = std::max({s.Y[0], s.Y[1], s.Y[2]});
    // pixel centres at 16 p + 8
    s.x0 = std::max<int64_t>(0, -floor_div(-(mnx - 8), 16));
    s.x1 = std::min<int64_t>(int64_t(W) - 1, floor_div(mxx - 8, 16));
    s.y0 = std::max<int64_t>(0, -floor_div(-(mny - 8), 16));
    s.y1 = std::min<int64_t>(int64_t(H) - 1, floor_div(mxy - 8, 16));
    return s.x0 <= s.x1 && s.y0 <= s.y1;
}

// a clipped polygon's fan triangle, FP64 clip coordinates
bool snap_tri(const V4& a, const V4& b, const V4& c, uint32_t W, uint32_t H, SnapTri& s) {
    const V4* v[3] = {&a, &b, &c};
    for (int i = 0; i < 3; ++i) {
        if (!(v[i]->w > 0.0)) return false;
        double nx = v[i]->x / v[i]->w, ny = v[i]->y / v[i]->w, nz = v[i]->z / v[i]->w;
        s.X[i] = std::llrint((nx + 1.0) * (8.0 * double(W)));
        s.Y[i] = std::llrint((ny + 1.0) * (8.0 * double(H)));
        s.Z[i] = nz;
    }
    return snap_finish(s, W, H);
}

// The common case, a triangle inside the clip volume: clip coordinates in FP32 with the FP32-rounded matrix
// (each product and sum rounded in order), division by w unless w == 1, snap in FP32; FP64 only in the plane.
struct V4f {
    float x, y, z, w;
};
inline float frow(const float* r, float x, float y, float z) {
    float a = r[0] * x;
    float b = r[1] * y;
    float c = r[2] * z;
    float t = a + b;
    t = t + c;
    return t + r[3];
}
inline bool inside_f(const V4f& v) {
    const float g = 16.0f * v.w;
    return v.z >= 0.0f && v.w - v.z >= 0.0f && g - v.x >= 0.0f && v.x + g >= 0.0f && g - v.y >= 0.0f &&
           v.y + g >= 0.0f;
}
inline float persp_div_f(float x, float w) { return w == 1.0f ? x : x / w; }
bool snap_tri_f(const V4f v[3], uint32_t W, uint32_t H, SnapTri& s) {
    const float sw = 8.0f * float(W), sh = 8.0f * float(H);
    for (int i = 0; i < 3; ++i) {
        if (!(v[i].w > 0.0f)) return false;
        const float nx = persp_div_f(v[i].x, v[i].w) + 1.0f, ny = persp_div_f(v[i].y, v[i].w) + 1.0f;
        s.X[i] = std::llrint(nx * sw);
        s.Y[i] = std::llrint(ny * sh);
        s.Z[i] = double(persp_div_f(v[i].z, v[i].w));
    }
    s.f32z = true;
    return snap_finish(s, W, H);
}

void raster_tri(const SnapTri& s, uint32_t tri, uint32_t W, int64_t row_lo, int64_t row_hi, uint64_t* keys) {
    int64_t y0 = std::max(s.y0, row_lo), y1 = std::min(s.y1, row_hi - 1);
    for (int64_t py = y0; py <= y1; ++py) {
        int64_t Py = 16 * py + 8;
        for (int64_t px = s.x0; px <= s.x1; ++px) {
            int64_t Px = 16 * px + 8;
            int64_t e0 = (s.X[2] - s.X[1]) * (Py - s.Y[1]) - (s.Y[2] - s.Y[1]) * (Px - s.X[1]);
            int64_t e1 = (s.X[0] - s.X[2]) * (Py - s.Y[2]) - (s.Y[0] - s.Y[2]) * (Px - s.X[2]);
            int64_t e2 = (s.X[1] - s.X[0]) * (Py - s.Y[0]) - (s.Y[1] - s.Y[0]) * (Px - s.X[0]);
            if (e0 < 0 || e1 < 0 || e2 < 0) continue;
            float ta = s.a * float(Px - s.X[0]);
            float zf = s.z0 + ta;
            float tb = s.b * float(Py - s.Y[0]);
            zf = zf + tb;
            if (!(zf > 0.0f)) zf = 0.0f;  // also maps -0 and NaN to +0
            if (zf > 1.0f) zf = 1.0f;
            uint64_t key = (uint64_t(float_bits(zf)) << 32) | tri;
            uint64_t& k = keys[uint64_t(py) * W + uint64_t(px)];
            if (key < k) k = key;
        }
    }
}

// ---------------- shared small math ----------------

template <class T>
struct Vec3 {
    T x, y, z;
};
template <class T>
inline Vec3<T> vsub(Vec3<T> a, Vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T>
inline Vec3<T> vadd(Vec3<T> a, Vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T>
inline Vec3<T> vmul(Vec3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T>
inline T vdot(Vec3<T> a, Vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
inline Vec3<T> vcross(Vec3<T> a, Vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T>
inline Vec3<T> vnorm(Vec3<T> a) {
    T l = std::sqrt(vdot(a, a));
    return l > T(0) ? vmul(a, T(1) / l) : a;
}

// make_coord_space, Shader/Lighting/indirect.frag:71-86 (h takes 1 in the smallest-magnitude component)
template <class T>
void make_coord_space(Vec3<T> n, Vec3<T>& x, Vec3<T>& y, Vec3<T>& z) {
    z = n;
    Vec3<T> h = z;
    using std::abs;
    if (abs(h.x) <= abs(h.y) && abs(h.x) <= abs(h.z))
        h.x = T(1);
    else if (abs(h.y) <= abs(h.x) && abs(h.y) <= abs(h.z))
        h.y = T(1);
    else
        h.z = T(1);
    z = vnorm(z);
    y = vnorm(vcross(h, z));
    x = vnorm(vcross(z, y));
}

uint16_t f2h(double x) {
    uint16_t sign = std::signbit(x) ? 0x8000 : 0;
    double a = std::fabs(x);
    if (std::isnan(x)) return 0x7e00;
    if (a >= 65520.0) return sign | 0x7c00;
    if (a < std::ldexp(1.0, -14)) {
        double q = std::nearbyint(a * std::ldexp(1.0, 24));
        return sign | uint16_t(q);
    }
    int e;
    std::frexp(a, &e);
    int E = e - 1;
    double q = std::nearbyint(a * std::ldexp(1.0, 10 - E));
    if (q >= 2048.0) {
        q = 1024.0;
        E += 1;
    }
    if (E + 15 >= 31) return sign | 0x7c00;
    return sign | uint16_t(((E + 15) << 10) | (int(q) - 1024));
}

double h2f(uint16_t h) {
    int s = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
    double v;
    if (e == 0)
        v = std::ldexp(double(m), -24);
    else if (e == 31)
        v = m ? NAN : INFINITY;
    else
        v = std::ldexp(double(m + 1024), e - 25);
    return s ? -v : v;
}

template <class T>
Vec3<T> oct_decode(uint32_t packed) {
    T x = T(h2f(uint16_t(packed & 0xffff)));
    T y = T(h2f(uint16_t(packed >> 16)));
    Vec3<T> v{x, y, T(1) - std::abs(x) - std::abs(y)};
    if (v.z < T(0)) {
        T ox = v.x, oy = v.y;
        v.x = (T(1) - std::abs(oy)) * (ox >= T(0) ? T(1) : T(-1));
        v.y = (T(1) - std::abs(ox)) * (oy >= T(0) ? T(1) : T(-1));
    }
    return vnorm(v);
}

uint32_t oct_encode_d(Vec3<double> n) {
    double s = std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z);
    double x = n.x / s, y = n.y / s;
    if (n.z < 0.0) {
        double ox = x, oy = y;
        x = (1.0 - std::fabs(oy)) * (ox >= 0.0 ? 1.0 : -1.0);
        y = (1.0 - std::fabs(ox)) * (oy >= 0.0 ? 1.0 : -1.0);
    }
    return uint32_t(f2h(x)) | (uint32_t(f2h(y)) << 16);
}

bool inverse4(const double* m, double* inv) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? m[r * 4 + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        if (a[p][c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < 8; ++k) std::swap(a[p][k], a[c][k]);
        double iv = 1.0 / a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] *= iv;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[r * 4 + c] = a[r][c + 4];
    return true;
}

// ---------------- voxelization ----------------

struct FixTri {
    int64_t q[3][3];
    int64_t n[3];
    int64_t lo[3], hi[3];  // voxel range (inclusive)
};

bool fix_tri(const f184gi_grid_frame& fr, uint32_t dim, const float* p, FixTri& t) {
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(p[i])) return false;  // triangles with a NaN or infinite coordinate are skipped
    for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
            double d = double(p[v * 3 + a]) - fr.origin[a];
            double s = d * fr.inv_voxel_fixed;
            int64_t q = std::llrint(s);
            if (q >= kMaxFixed || q <= -kMaxFixed) return false;
            t.q[v][a] = q;
        }
    int64_t e0[3], e1[3];
    for (int a = 0; a < 3; ++a) {
        e0[a] = t.q[1][a] - t.q[0][a];
        e1[a] = t.q[2][a] - t.q[0][a];
    }
    t.n[0] = e0[1] * e1[2] - e0[2] * e1[1];
    t.n[1] = e0[2] * e1[0] - e0[0] * e1[2];
    t.n[2] = e0[0] * e1[1] - e0[1] * e1[0];
    if (t.n[0] == 0 && t.n[1] == 0 && t.n[2] == 0) return false;
    for (int a = 0; a < 3; ++a) {
        int64_t mn = std::min({t.q[0][a], t.q[1][a], t.q[2][a]});
        int64_t mx = std::max({t.q[0][a], t.q[1][a], t.q[2][a]});
        // voxel i (box [256 i, 256 i + 256]) touches [mn, mx] iff 256 i <= mx and 256 i + 256 >= mn
        t.lo[a] = std::max<int64_t>(0, -floor_div(-(mn - kVoxelFixed), kVoxelFixed));
        t.hi[a] = std::min<int64_t>(int64_t(dim) - 1, floor_div(mx, kVoxelFixed));
        if (t.lo[a] > t.hi[a]) return false;
    }
    return true;
}

inline int64_t iabs(int64_t x) { return x < 0 ? -x : x; }

// Closed-set triangle / voxel overlap by the separating-axis theorem (Akenine-Moller), exact in int64.
bool tri_box_overlap(const FixTri& t, int64_t i, int64_t j, int64_t k) {
    const int64_t c[3] = {i * kVoxelFixed + kHalfVoxel, j * kVoxelFixed + kHalfVoxel, k * kVoxelFixed + kHalfVoxel};
    int64_t v[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) v[a][b] = t.q[a][b] - c[b];
    const int64_t h = kHalfVoxel;
    // box axes
    for (int b = 0; b < 3; ++b) {
        int64_t mn = std::min({v[0][b], v[1][b], v[2][b]}), mx = std::max({v[0][b], v[1][b], v[2][b]});
        if (mn > h || mx < -h) return false;
    }
    // triangle plane
    {
        int64_t s = t.n[0] * v[0][0] + t.n[1] * v[0][1] + t.n[2] * v[0][2];
        int64_t r = h * (iabs(t.n[0]) + iabs(t.n[1]) + iabs(t.n[2]));
        if (s > r || s < -r) return false;
    }
    // edge x axis
    for (int e = 0; e < 3; ++e) {
        int64_t ed[3];
        for (int b = 0; b < 3; ++b) ed[b] = v[(e + 1) % 3][b] - v[e][b];
        for (int ax = 0; ax < 3; ++ax) {
            int64_t a[3] = {0, 0, 0};
            // a = ed x unit(ax)
            if (ax == 0) { a[1] = ed[2]; a[2] = -ed[1]; }
            if (ax == 1) { a[0] = -ed[2]; a[2] = ed[0]; }
            if (ax == 2) { a[0] = ed[1]; a[1] = -ed[0]; }
            int64_t p0 = a[0] * v[0][0] + a[1] * v[0][1] + a[2] * v[0][2];
            int64_t p1 = a[0] * v[1][0] + a[1] * v[1][1] + a[2] * v[1][2];
            int64_t p2 = a[0] * v[2][0] + a[1] * v[2][1] + a[2] * v[2][2];
            int64_t r = h * (iabs(a[0]) + iabs(a[1]) + iabs(a[2]));
            int64_t mn = std::min({p0, p1, p2}), mx = std::max({p0, p1, p2});
            if (mn > r || mx < -r) return false;
        }
    }
    return true;
}

// Shadow visibility of the centre of voxel (i, j, k), FP32 in this exact operation order (the decision must
// not depend on the arithmetic precision of the caller):
//   v_r = ((base_r + i s_r0) + j s_r1) + k s_r2,  texel = floor((v + 1) * res/2),  lit = z - bias <= depth
inline float vox_light(const float* lv, float fi, float fj, float fk) {
    float a = fi * lv[1];
    float s = lv[0] + a;
    float b = fj * lv[2];
    s = s + b;
    float c = fk * lv[3];
    return s + c;
}

bool shade_voxel(const f184gi_grid_frame& fr, uint32_t res, const float* shadow, int64_t i, int64_t j, int64_t k) {
    float fi = float(i), fj = float(j), fk = float(k);
    float x = vox_light(fr.light_vox + 0, fi, fj, fk);
    float y = vox_light(fr.light_vox + 4, fi, fj, fk);
    float z = vox_light(fr.light_vox + 8, fi, fj, fk);
    float half = 0.5f * float(res);
    float tx = std::floor((x + 1.0f) * half), ty = std::floor((y + 1.0f) * half);
    if (!(tx >= 0.0f && ty >= 0.0f && tx < float(res) && ty < float(res))) return true;
    float sd = shadow[uint64_t(ty) * res + uint64_t(tx)];
    float zb = z - fr.shadow_bias_f;
    return zb <= sd;
}

template <class T>
T albedo_lin(uint32_t byte) {
    return T(std::pow(double(byte) / 255.0, 2.2));
}
template <>
float albedo_lin<float>(uint32_t byte) {
    return std::pow(float(byte) / 255.0f, 2.2f);
}

template <class T>
int voxelize_impl(const f184gi_grid_frame* frame, uint32_t dim, uint32_t res, const float* tri,
                  const uint32_t* albedo, uint64_t ntris, const f184gi_light* light, const float* shadow,
                  T* rgba, uint32_t* counts_out, int nthreads) {
    if (!frame || !tri || !albedo || !light || !shadow || !rgba || dim == 0) return -1;
    const f184gi_grid_frame& fr = *frame;
    const uint64_t nvox = uint64_t(dim) * dim * dim;
    std::vector<FixTri> ft(ntris);
    std::vector<uint8_t> ok(ntris);
    std::vector<T> w(ntris * 3);
    Vec3<T> wi{T(-fr.light_dir[0]), T(-fr.light_dir[1]), T(-fr.light_dir[2])};
    parallel_for(0, int64_t(ntris), nthreads, [&](int64_t b, int64_t e) {
        for (int64_t t = b; t < e; ++t) {
            ok[t] = fix_tri(fr, dim, tri + t * 9, ft[t]);
            const float* p = tri + t * 9;
            Vec3<T> p0{T(p[0]), T(p[1]), T(p[2])}, p1{T(p[3]), T(p[4]), T(p[5])}, p2{T(p[6]), T(p[7]), T(p[8])};
            Vec3<T> n = vcross(vsub(p1, p0), vsub(p2, p0));
            T len = std::sqrt(vdot(n, n));
            T cosv = len > T(0) ? std::abs(vdot(wi, n)) / len : T(0);
            uint32_t a = albedo[t];
            for (int c = 0; c < 3; ++c) w[t * 3 + c] = cosv * albedo_lin<T>((a >> (8 * c)) & 255u);
        }
    });
    std::vector<T> sum(nvox * 3, T(0));
    std::vector<uint32_t> cnt(nvox, 0);
    // z-slab partition: each thread owns whole voxels, so every voxel sums in triangle order
    parallel_for(0, int64_t(dim), nthreads, [&](int64_t kb, int64_t ke) {
        for (uint64_t t = 0; t < ntris; ++t) {
            if (!ok[t]) continue;
            const FixTri& f = ft[t];
            int64_t k0 = std::max(f.lo[2], kb), k1 = std::min(f.hi[2], ke - 1);
            for (int64_t k = k0; k <= k1; ++k)
                for (int64_t j = f.lo[1]; j <= f.hi[1]; ++j)
                    for (int64_t i = f.lo[0]; i <= f.hi[0]; ++i) {
                        if (!tri_box_overlap(f, i, j, k)) continue;
                        uint64_t idx = (uint64_t(k) * dim + uint64_t(j)) * dim + uint64_t(i);
                        cnt[idx] += 1;
                        for (int c = 0; c < 3; ++c) sum[idx * 3 + c] += w[t * 3 + c];
                    }
        }
    });
    parallel_for(0, int64_t(dim), nthreads, [&](int64_t kb, int64_t ke) {
        for (int64_t k = kb; k < ke; ++k)
            for (int64_t j = 0; j < int64_t(dim); ++j)
                for (int64_t i = 0; i < int64_t(dim); ++i) {
                    uint64_t idx = (uint64_t(k) * dim + uint64_t(j)) * dim + uint64_t(i);
                    T* o = rgba + idx * 4;
                    if (cnt[idx] == 0) {
                        o[0] = o[1] = o[2] = o[3] = T(0);
                        continue;
                    }
                    T lit = shade_voxel(fr, res, shadow, i, j, k) ? T(1) : T(0);
                    T inv = T(1) / T(cnt[idx]);
                    for (int c = 0; c < 3; ++c) o[c] = T(light->luminance[c]) * lit * (sum[idx * 3 + c] * inv);
                    o[3] = T(1);
                }
    });
    if (counts_out) std::memcpy(counts_out, cnt.data(), nvox * 4);
    return 0;
}

// ---------------- mips ----------------

template <class T>
void mip_level(const T* src, uint32_t sd, T* dst, int nthreads) {
    uint32_t dd = sd / 2;
    parallel_for(0, int64_t(dd), nthreads, [&](int64_t kb, int64_t ke) {
        for (int64_t k = kb; k < ke; ++k)
            for (uint32_t j = 0; j < dd; ++j)
                for (uint32_t i = 0; i < dd; ++i) {
                    T acc[4] = {T(0), T(0), T(0), T(0)};
                    for (int dz = 0; dz < 2; ++dz)
                        for (int dy = 0; dy < 2; ++dy)
                            for (int dx = 0; dx < 2; ++dx) {
                                uint64_t s = ((uint64_t(2 * k + dz) * sd) + (2 * j + dy)) * sd + (2 * i + dx);
                                for (int c = 0; c < 4; ++c) acc[c] += src[s * 4 + c];
                            }
                    uint64_t d = ((uint64_t(k) * dd) + j) * dd + i;
                    for (int c = 0; c < 4; ++c) dst[d * 4 + c] = acc[c] * T(0.125);
                }
    });
}

template <class T>
int mip_impl(T* chain, uint32_t dim, uint32_t levels, int nthreads) {
    if (!chain || levels == 0 || (dim >> (levels - 1)) == 0) return -1;
    uint64_t off = 0;
    for (uint32_t l = 1; l < levels; ++l) {
        uint32_t sd = dim >> (l - 1);
        T* src = chain + off;
        off += uint64_t(sd) * sd * sd * 4;
        mip_level(src, sd, chain + off, nthreads);
    }
    return 0;
}

// Anisotropic: direction d in (+x,-x,+y,-y,+z,-z) composites the two children along the axis front to
// back (front = the child a cone travelling along d meets first) and averages the four columns.
template <class T>
void mip_aniso_level(const T* const src_dir[6], uint32_t sd, T* const dst_dir[6], int nthreads) {
    uint32_t dd = sd / 2;
    parallel_for(0, int64_t(dd), nthreads, [&](int64_t kb, int64_t ke) {
        for (int64_t k = kb; k < ke; ++k)
            for (uint32_t j = 0; j < dd; ++j)
                for (uint32_t i = 0; i < dd; ++i) {
                    uint64_t d = ((uint64_t(k) * dd) + j) * dd + i;
                    for (int dir = 0; dir < 6; ++dir) {
                        const T* src = src_dir[dir];
                        int axis = dir / 2;
                        bool neg = dir & 1;
                        T acc[4] = {T(0), T(0), T(0), T(0)};
                        for (int u = 0; u < 2; ++u)
                            for (int v = 0; v < 2; ++v) {
                                int off_f[3], off_b[3];
                                // (u, v) span the two axes other than `axis`
                                int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
                                off_f[axis] = neg ? 1 : 0;
                                off_b[axis] = neg ? 0 : 1;
                                off_f[o1] = off_b[o1] = u;
                                off_f[o2] = off_b[o2] = v;
                                uint64_t sf = ((uint64_t(2 * k + off_f[2]) * sd) + (2 * j + off_f[1])) * sd + (2 * i + off_f[0]);
                                uint64_t sb = ((uint64_t(2 * k + off_b[2]) * sd) + (2 * j + off_b[1])) * sd + (2 * i + off_b[0]);
                                const T* f = src + sf * 4;
                                const T* b = src + sb * 4;
                                T tr = T(1) - f[3];
                                for (int c = 0; c < 4; ++c) acc[c] += f[c] + tr * b[c];
                            }
                        for (int c = 0; c < 4; ++c) dst_dir[dir][d * 4 + c] = acc[c] * T(0.25);
                    }
                }
    });
}

template <class T>
int mip_aniso_impl(T* chain, uint32_t dim, uint32_t levels, int nthreads) {
    if (!chain || levels == 0 || (dim >> (levels - 1)) == 0) return -1;
    uint64_t off = uint64_t(dim) * dim * dim * 4;
    const T* src[6];
    for (int d = 0; d < 6; ++d) src[d] = chain;
    for (uint32_t l = 1; l < levels; ++l) {
        uint32_t sd = dim >> (l - 1), dd = sd / 2;
        uint64_t vol = uint64_t(dd) * dd * dd * 4;
        T* dst[6];
        for (int d = 0; d < 6; ++d) dst[d] = chain + off + vol * d;
        mip_aniso_level(src, sd, dst, nthreads);
        for (int d = 0; d < 6; ++d) src[d] = dst[d];
        off += vol * 6;
    }
    return 0;
}

// ---------------- cone trace ----------------

f184gi_cone_params default_params() {
    f184gi_cone_params p;
    p.diffuse_cones = 5;
    p.diffuse_tan_half = 0.57735026918962576f;  // tan(30 deg)
    p.diffuse_tilt_deg = 60.0f;
    p.step_factor = 0.5f;
    p.max_distance = 0.0f;
    p.alpha_stop = 1.0f;
    p.start_offset = 1.0f;
    p.min_spec_tan_half = 0.05f;
    p.specular = 1;
    p.pad = 0;
    return p;
}

template <class T>
struct Chain {
    const T* base;
    uint32_t dim, levels;
    bool aniso;
    uint64_t off[16];  // level offsets (aniso: first direction volume)
};

template <class T>
Chain<T> make_chain(const T* base, uint32_t dim, uint32_t levels, bool aniso) {
    Chain<T> c{base, dim, levels, aniso, {}};
    uint64_t o = 0;
    for (uint32_t l = 0; l < levels && l < 16; ++l) {
        c.off[l] = o;
        uint64_t d = dim >> l;
        o += d * d * d * 4 * ((aniso && l > 0) ? 6 : 1);
    }
    return c;
}

template <class T>
void tri_sample(const T* vol, int64_t d, Vec3<T> x, T inv_scale, T out[4]) {
    T u[3] = {x.x * inv_scale - T(0.5), x.y * inv_scale - T(0.5), x.z * inv_scale - T(0.5)};
    int64_t i0[3];
    T f[3];
    for (int a = 0; a < 3; ++a) {
        T fl = std::floor(u[a]);
        i0[a] = int64_t(fl);
        f[a] = u[a] - fl;
    }
    out[0] = out[1] = out[2] = out[3] = T(0);
    for (int dz = 0; dz < 2; ++dz) {
        int64_t z = i0[2] + dz;
        if (z < 0 || z >= d) continue;
        T wz = dz ? f[2] : T(1) - f[2];
        for (int dy = 0; dy < 2; ++dy) {
            int64_t y = i0[1] + dy;
            if (y < 0 || y >= d) continue;
            T wy = dy ? f[1] : T(1) - f[1];
            for (int dx = 0; dx < 2; ++dx) {
                int64_t xx = i0[0] + dx;
                if (xx < 0 || xx >= d) continue;
                T wx = dx ? f[0] : T(1) - f[0];
                T w = wx * wy * wz;
                const T* v = vol + (((uint64_t(z) * d) + uint64_t(y)) * d + uint64_t(xx)) * 4;
                for (int c = 0; c < 4; ++c) out[c] += w * v[c];
            }
        }
    }
}

template <class T>
void level_sample(const Chain<T>& ch, uint32_t l, Vec3<T> x, Vec3<T> dir, T out[4]) {
    int64_t d = ch.dim >> l;
    T inv_scale = T(std::ldexp(1.0, -int(l)));
    if (!ch.aniso || l == 0) {
        tri_sample(ch.base + ch.off[l], d, x, inv_scale, out);
        return;
    }
    uint64_t vol = uint64_t(d) * d * d * 4;
    T w[3] = {dir.x * dir.x, dir.y * dir.y, dir.z * dir.z};
    int sel[3] = {dir.x >= T(0) ? 0 : 1, dir.y >= T(0) ? 2 : 3, dir.z >= T(0) ? 4 : 5};
    out[0] = out[1] = out[2] = out[3] = T(0);
    for (int a = 0; a < 3; ++a) {
        T s[4];
        tri_sample(ch.base + ch.off[l] + vol * sel[a], d, x, inv_scale, s);
        for (int c = 0; c < 4; ++c) out[c] += w[a] * s[c];
    }
}

// cnt (optional): cnt[0] += steps, cnt[1] += level samples (one or two per step)
template <class T>
void cone(const Chain<T>& ch, Vec3<T> o, Vec3<T> dir, T tan_half, const f184gi_cone_params& p, T tmax,
          T out[4], uint64_t* cnt = nullptr) {
    T c[3] = {T(0), T(0), T(0)}, alpha = T(0);
    // FP64: t accumulates plainly (the definition).  FP32 (the device arithmetic): the distance is the pair
    // t + tl advanced with error-free sums, so long marches of small steps do not drift.
    constexpr bool kPair = std::is_same<T, float>::value;
    T t = T(p.start_offset), tl = T(0);
    const T dimf = T(ch.dim);
    const T maxl = T(ch.levels - 1);
    const T d2 = T(2) * tan_half;
    while (t < tmax || (t == tmax && tl <= T(0))) {
        T diam = kPair ? std::max(T(1), std::fma(d2, t, d2 * tl)) : std::max(T(1), T(2) * t * tan_half);
        T lvl = std::min(std::max(std::log2(diam), T(0)), maxl);
        Vec3<T> x = kPair ? Vec3<T>{std::fma(dir.x, t, std::fma(dir.x, tl, o.x)), std::fma(dir.y, t, std::fma(dir.y, tl, o.y)),
                                    std::fma(dir.z, t, std::fma(dir.z, tl, o.z))}
                          : vadd(o, vmul(dir, t));
        T m = T(2) * diam;
        if (x.x < -m || x.y < -m || x.z < -m || x.x > dimf + m || x.y > dimf + m || x.z > dimf + m) break;
        T fl = std::floor(lvl);
        uint32_t l0 = uint32_t(fl);
        T f = lvl - fl;
        if (cnt) {
            cnt[0] += 1;
            cnt[1] += (f > T(0) && l0 + 1 < ch.levels) ? 2 : 1;
        }
        T s[4];
        level_sample(ch, l0, x, dir, s);
        if (f > T(0) && l0 + 1 < ch.levels) {
            T s1[4];
            level_sample(ch, l0 + 1, x, dir, s1);
            for (int k = 0; k < 4; ++k) s[k] = s[k] + f * (s1[k] - s[k]);
        }
        T tr = T(1) - alpha;
        for (int k = 0; k < 3; ++k) c[k] += tr * s[k];
        alpha += tr * s[3];
        if (alpha >= T(p.alpha_stop)) break;
        const T step = T(p.step_factor) * diam;
        if (kPair) {
            const T ts = t + step, tb = ts - t;
            tl += (t - (ts - tb)) + (step - tb);
            t = ts;
        } else {
            t += step;
        }
    }
    out[0] = c[0];
    out[1] = c[1];
    out[2] = c[2];
    out[3] = alpha;
}

// The FP32 path's pixel set-up and cone march, in the device's sequence (every operation rounded on its own).
// Set-up in float-float (Knuth's two-sum and the FMA two-product are exact): the cone origin in voxel units to
// ~1e-9 voxel, split into an integer voxel oi and an offset of.  The march keeps the sample point as oi + x with x
// small, and forms each level coordinate as (oi 2^-l - 0.5) split exactly into integer + fraction, plus x 2^-l:
// the tap weights then carry the precision of x, not of the grid-sized coordinate.
inline FF32 ff_row(const float* h, const float* l, FF32 x, FF32 y, FF32 z) {
    FF32 s = ff_add(ff_mul(FF32{h[0], l[0]}, x), ff_mul(FF32{h[1], l[1]}, y));
    s = ff_add(s, ff_mul(FF32{h[2], l[2]}, z));
    return ff_add(s, FF32{h[3], l[3]});
}
inline FF32 ff_ndc(uint32_t k, uint32_t n) {
    const float num = float(2u * k + 1u), den = float(n);
    const float q = num / den;
    const float ql = std::fma(-q, den, num) / den;
    return ff_add(FF32{q, ql}, FF32{-1.0f, 0.0f});
}

// 8-tap sample of one volume of level l at oi + x (p = oi + x rounded to FP32), added to out scaled by `scale`.
// Level 0 splits its coordinate exactly as (oi - 1) + (x + 0.5), so the tap fraction keeps the precision of x;
// coarser levels take u + 1 = p 2^-l + 0.5 in FP32 (the rounding of p shrinks by 2^-l there).
void tri_sample_rel(const float* vol, int64_t d, uint32_t l, const float oi[3], const float x[3], const float p[3],
                    float scale, float out[4]) {
    const float s = std::ldexp(1.0f, -int(l));
    int64_t i0[3];
    float f[3];
    for (int a = 0; a < 3; ++a) {
        if (l == 0) {
            const float v = x[a] + 0.5f;
            const float fl = std::floor(v);
            i0[a] = int64_t((oi[a] - 1.0f) + fl);
            f[a] = v - fl;
        } else {  // u + 1 = p 2^-l + 0.5: its floor is the first tap + 1
            const float u1 = std::fma(p[a], s, 0.5f);
            const float fl = std::floor(u1);
            i0[a] = int64_t(fl) - 1;
            f[a] = u1 - fl;
        }
    }
    for (int dz = 0; dz < 2; ++dz) {
        const int64_t z = i0[2] + dz;
        if (z < 0 || z >= d) continue;
        const float wz = (dz ? f[2] : 1.0f - f[2]) * scale;
        for (int dy = 0; dy < 2; ++dy) {
            const int64_t y = i0[1] + dy;
            if (y < 0 || y >= d) continue;
            const float wyz = (dy ? f[1] : 1.0f - f[1]) * wz;
            for (int dx = 0; dx < 2; ++dx) {
                const int64_t xx = i0[0] + dx;
                if (xx < 0 || xx >= d) continue;
                const float w = (dx ? f[0] : 1.0f - f[0]) * wyz;
                const float* v = vol + (((uint64_t(z) * d) + uint64_t(y)) * d + uint64_t(xx)) * 4;
                for (int c = 0; c < 4; ++c) out[c] = std::fma(w, v[c], out[c]);
            }
        }
    }
}

void level_sample_rel(const Chain<float>& ch, uint32_t l, const float oi[3], const float x[3], const float p[3],
                      Vec3<float> dir, float scale, float out[4]) {
    const int64_t d = ch.dim >> l;
    if (!ch.aniso || l == 0) {
        tri_sample_rel(ch.base + ch.off[l], d, l, oi, x, p, scale, out);
        return;
    }
    const uint64_t vol = uint64_t(d) * d * d * 4;
    const float w[3] = {dir.x * dir.x * scale, dir.y * dir.y * scale, dir.z * dir.z * scale};
    const int sel[3] = {dir.x >= 0.0f ? 0 : 1, dir.y >= 0.0f ? 2 : 3, dir.z >= 0.0f ? 4 : 5};
    for (int a = 0; a < 3; ++a) {
        float sa[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        tri_sample_rel(ch.base + ch.off[l] + vol * sel[a], d, l, oi, x, p, 1.0f, sa);
        for (int c = 0; c < 4; ++c) out[c] = std::fma(w[a], sa[c], out[c]);
    }
}

// The FP32 cone from the split origin oi + of (the device's march): quadrilinear as (1 - f) level l0 + f level l0+1
// with the level weights folded into the tap weights; distance t + tl advanced with error-free sums.
void cone_rel(const Chain<float>& ch, const float oi[3], const float of[3], Vec3<float> dir, float tan_half,
              const f184gi_cone_params& p, float tmax, float out[4], uint64_t* cnt) {
    float c[3] = {0.0f, 0.0f, 0.0f}, alpha = 0.0f;
    float t = p.start_offset, tl = 0.0f;
    const float dimf = float(ch.dim), maxl = float(ch.levels - 1), d2 = 2.0f * tan_half;
    const float dv[3] = {dir.x, dir.y, dir.z};
    while (t < tmax || (t == tmax && tl <= 0.0f)) {
        const float diam = std::max(1.0f, std::fma(d2, t, d2 * tl));
        const float lvl = std::min(std::max(std::log2(diam), 0.0f), maxl);
        float x[3], pa[3];
        bool outside = false;
        const float m = 2.0f * diam;
        for (int a = 0; a < 3; ++a) {
            x[a] = std::fma(dv[a], t, std::fma(dv[a], tl, of[a]));
            pa[a] = oi[a] + x[a];
            outside = outside || pa[a] < -m || pa[a] > dimf + m;
        }
        if (outside) break;
        const float fl = std::floor(lvl);
        const uint32_t l0 = uint32_t(fl);
        const float f = lvl - fl;
        const bool two = f > 0.0f && l0 + 1 < ch.levels;
        if (cnt) {
            cnt[0] += 1;
            cnt[1] += two ? 2 : 1;
        }
        float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        level_sample_rel(ch, l0, oi, x, pa, dir, two ? 1.0f - f : 1.0f, s);
        if (two) level_sample_rel(ch, l0 + 1, oi, x, pa, dir, f, s);
        const float tr = 1.0f - alpha;
        for (int k = 0; k < 3; ++k) c[k] += tr * s[k];
        alpha += tr * s[3];
        if (alpha >= p.alpha_stop) break;
        const float step = p.step_factor * diam;
        const float ts = t + step, tb = ts - t;
        tl += (t - (ts - tb)) + (step - tb);
        t = ts;
    }
    out[0] = c[0], out[1] = c[1], out[2] = c[2], out[3] = alpha;
}

// FP64: the definition (cone from the origin o); FP32: the device's march from the split origin
inline void trace_cone(const Chain<double>& ch, const float*, const float*, Vec3<double> o, Vec3<double> dir,
                       double tan_half, const f184gi_cone_params& p, double tmax, double out[4], uint64_t* cnt) {
    cone(ch, o, dir, tan_half, p, tmax, out, cnt);
}
inline void trace_cone(const Chain<float>& ch, const float* oi, const float* of, Vec3<float>, Vec3<float> dir,
                       float tan_half, const f184gi_cone_params& p, float tmax, float out[4], uint64_t* cnt) {
    cone_rel(ch, oi, of, dir, tan_half, p, tmax, out, cnt);
}

template <class T>
int trace_impl(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso, const T* chain,
               const float view[16], const float proj[16], uint32_t W, uint32_t H, const float* depth,
               const uint32_t* normal, const uint16_t* rough, const f184gi_cone_params* params, T* out,
               uint32_t row_begin, uint32_t row_end, int nthreads, uint64_t* counts = nullptr) {
    if (!frame || !chain || !view || !proj || !depth || !normal || !rough || !out) return -1;
    f184gi_cone_params p = default_params();
    if (params) p = *params;
    double V[16], P[16], IV[16], IP[16];
    for (int i = 0; i < 16; ++i) {
        V[i] = view[i];
        P[i] = proj[i];
    }
    if (!inverse4(V, IV) || !inverse4(P, IP)) return -1;
    T iv[16], ip[16];
    for (int i = 0; i < 16; ++i) {
        iv[i] = T(IV[i]);
        ip[i] = T(IP[i]);
    }
    // the FP32 path's float-float set-up: IP, IV (rows 0..2), the grid origin and scale as FP32 pairs
    float ip_h[16], ip_l[16], iv_h[12], iv_l[12], org_h[3], org_l[3];
    for (int k = 0; k < 16; ++k) ip_h[k] = float(IP[k]), ip_l[k] = float(IP[k] - double(ip_h[k]));
    for (int k = 0; k < 12; ++k) iv_h[k] = float(IV[k]), iv_l[k] = float(IV[k] - double(iv_h[k]));
    for (int a = 0; a < 3; ++a) org_h[a] = float(frame->origin[a]), org_l[a] = float(frame->origin[a] - double(org_h[a]));
    const double ivs_d = frame->inv_voxel_fixed * (1.0 / 256.0);
    const float ivs_h = float(ivs_d), ivs_l = float(ivs_d - double(ivs_h));
    Chain<T> ch = make_chain(chain, dim, levels, aniso != 0);
    const T vs = T(frame->voxel_size);
    const T inv_vs = T(1.0 / frame->voxel_size);
    const Vec3<T> org{T(frame->origin[0]), T(frame->origin[1]), T(frame->origin[2])};
    const T tmax = p.max_distance > 0 ? T(p.max_distance) : T(double(dim) * std::sqrt(3.0));
    const double tilt = double(p.diffuse_tilt_deg) * M_PI / 180.0;
    const T ct = T(std::cos(tilt)), st = T(std::sin(tilt));
    const uint64_t npix = uint64_t(W) * H;
    (void)vs;
    Vec3<T> eye{iv[3], iv[7], iv[11]};
    // pixels of rows [row_begin, row_end), split evenly over the threads
    const int64_t p_begin = int64_t(row_begin) * W, p_end = int64_t(std::min(row_end, H)) * W;
    parallel_for(p_begin, p_end, nthreads, [&](int64_t pb, int64_t pe) {
        uint64_t lc[2] = {0, 0};
        uint64_t* cnt = counts ? lc : nullptr;
        for (int64_t pix = pb; pix < pe; ++pix) {
            {
                const int64_t py = pix / W;
                const uint32_t px = uint32_t(pix % W);
                uint64_t pi = uint64_t(pix);
                T* od = out + pi * 4;
                T* os = out + (npix + pi) * 4;
                for (int k = 0; k < 4; ++k) od[k] = os[k] = T(0);
                float dd = depth[pi];
                if (!(dd < 1.0f)) continue;
                T nx = (T(px) + T(0.5)) / T(W) * T(2) - T(1);
                T ny = (T(py) + T(0.5)) / T(H) * T(2) - T(1);
                T nz = T(dd);
                T vp[4];
                for (int r = 0; r < 4; ++r) vp[r] = ip[r * 4 + 0] * nx + ip[r * 4 + 1] * ny + ip[r * 4 + 2] * nz + ip[r * 4 + 3];
                Vec3<T> cs{vp[0] / vp[3], vp[1] / vp[3], vp[2] / vp[3]};
                float oi[3] = {0, 0, 0}, of[3] = {0, 0, 0};  // FP32 path: the split cone origin
                FF32 wpf[3] = {};
                if (std::is_same<T, float>::value) {
                    // the device arithmetic: position in float-float
                    const FF32 ndx = ff_ndc(px, W), ndy = ff_ndc(uint32_t(py), H), dzf = FF32{dd, 0.0f};
                    const FF32 vwf = ff_row(ip_h + 12, ip_l + 12, ndx, ndy, dzf);
                    const FF32 cxf = ff_div(ff_row(ip_h, ip_l, ndx, ndy, dzf), vwf);
                    const FF32 cyf = ff_div(ff_row(ip_h + 4, ip_l + 4, ndx, ndy, dzf), vwf);
                    const FF32 czf = ff_div(ff_row(ip_h + 8, ip_l + 8, ndx, ndy, dzf), vwf);
                    for (int r = 0; r < 3; ++r) wpf[r] = ff_row(iv_h + 4 * r, iv_l + 4 * r, cxf, cyf, czf);
                    cs = Vec3<T>{T(cxf.h), T(cyf.h), T(czf.h)};
                }
                Vec3<T> wp{iv[0] * cs.x + iv[1] * cs.y + iv[2] * cs.z + iv[3],
                           iv[4] * cs.x + iv[5] * cs.y + iv[6] * cs.z + iv[7],
                           iv[8] * cs.x + iv[9] * cs.y + iv[10] * cs.z + iv[11]};
                Vec3<T> nv = oct_decode<T>(normal[pi]);
                Vec3<T> nw = vnorm(Vec3<T>{iv[0] * nv.x + iv[1] * nv.y + iv[2] * nv.z,
                                           iv[4] * nv.x + iv[5] * nv.y + iv[6] * nv.z,
                                           iv[8] * nv.x + iv[9] * nv.y + iv[10] * nv.z});
                T r = T(h2f(rough[pi]));
                if (std::is_same<T, float>::value) wp = Vec3<T>{T(wpf[0].h), T(wpf[1].h), T(wpf[2].h)};
                Vec3<T> pv = vmul(vsub(wp, org), inv_vs);
                Vec3<T> o = vadd(pv, vmul(nw, T(p.start_offset)));
                if (std::is_same<T, float>::value) {
                    const float na[3] = {float(nw.x), float(nw.y), float(nw.z)};
                    for (int a = 0; a < 3; ++a) {
                        const FF32 pf = ff_mul(ff_add(wpf[a], FF32{-org_h[a], -org_l[a]}), FF32{ivs_h, ivs_l});
                        const float q = na[a] * p.start_offset;
                        const FF32 of2 = ff_add(pf, FF32{q, std::fma(na[a], p.start_offset, -q)});
                        oi[a] = std::floor(of2.h);
                        of[a] = (of2.h - oi[a]) + of2.l;
                    }
                }
                Vec3<T> bx, by, bz;
                make_coord_space(nw, bx, by, bz);
                T acc[4] = {T(0), T(0), T(0), T(0)};
                if (p.diffuse_cones >= 5) {
                    T c0[4];
                    trace_cone(ch, oi, of, o, bz, T(p.diffuse_tan_half), p, tmax, c0, cnt);
                    for (int k = 0; k < 4; ++k) acc[k] += T(0.25) * c0[k];
                    const T cphi[4] = {T(1), T(0), T(-1), T(0)}, sphi[4] = {T(0), T(1), T(0), T(-1)};
                    for (int s = 0; s < 4; ++s) {
                        Vec3<T> side = vadd(vmul(bx, cphi[s]), vmul(by, sphi[s]));
                        Vec3<T> d = vnorm(vadd(vmul(bz, ct), vmul(side, st)));
                        T cs4[4];
                        trace_cone(ch, oi, of, o, d, T(p.diffuse_tan_half), p, tmax, cs4, cnt);
                        for (int k = 0; k < 4; ++k) acc[k] += T(0.1875) * cs4[k];
                    }
                } else {
                    trace_cone(ch, oi, of, o, bz, T(p.diffuse_tan_half), p, tmax, acc, cnt);
                }
                for (int k = 0; k < 4; ++k) od[k] = acc[k];
                if (p.specular) {
                    Vec3<T> vdir = vnorm(vsub(wp, eye));
                    T dn = vdot(vdir, nw);
                    Vec3<T> rd = vnorm(vsub(vdir, vmul(nw, T(2) * dn)));
                    T th = std::max(r, T(p.min_spec_tan_half));
                    T sc[4];
                    trace_cone(ch, oi, of, o, rd, th, p, tmax, sc, cnt);
                    for (int k = 0; k < 4; ++k) os[k] = sc[k];
                }
            }
        }
        if (counts) {
            __atomic_fetch_add(&counts[0], lc[0], __ATOMIC_RELAXED);
            __atomic_fetch_add(&counts[1], lc[1], __ATOMIC_RELAXED);
        }
    });
    return 0;
}

}  // namespace

extern "C" {

int orc_grid_frame(const f184gi_bounds* b, uint32_t dim, const float light_dir[3], f184gi_grid_frame* out) {
    if (!b || !out || dim < 4 || !light_dir) return -1;
    std::memset(out, 0, sizeof(*out));
    double c[3], ext = 0.0;
    const float mn[3] = {b->min.x, b->min.y, b->min.z}, mx[3] = {b->max.x, b->max.y, b->max.z};
    for (int a = 0; a < 3; ++a) {
        double s = double(mn[a]) + double(mx[a]);
        c[a] = s * 0.5;
        double e = double(mx[a]) - double(mn[a]);
        if (e > ext) ext = e;
    }
    if (!(ext > 0.0)) ext = 1.0;
    double vs = ext / double(dim - 3);
    double half = vs * (double(dim) * 0.5);
    for (int a = 0; a < 3; ++a) out->origin[a] = c[a] - half;
    out->voxel_size = vs;
    out->inv_voxel_fixed = 256.0 / vs;
    // light frame
    double L[3] = {light_dir[0], light_dir[1], light_dir[2]};
    double l2 = L[0] * L[0];
    l2 = l2 + L[1] * L[1];
    l2 = l2 + L[2] * L[2];
    double len = std::sqrt(l2);
    if (!(len > 0.0)) return -1;
    double w[3] = {L[0] / len, L[1] / len, L[2] / len};
    double h[3] = {0.0, 0.0, 0.0};
    double ax = std::fabs(w[0]), ay = std::fabs(w[1]), az = std::fabs(w[2]);
    if (ax <= ay && ax <= az)
        h[0] = 1.0;
    else if (ay <= az)
        h[1] = 1.0;
    else
        h[2] = 1.0;
    double u[3] = {h[1] * w[2] - h[2] * w[1], h[2] * w[0] - h[0] * w[2], h[0] * w[1] - h[1] * w[0]};
    double ul = u[0] * u[0];
    ul = ul + u[1] * u[1];
    ul = ul + u[2] * u[2];
    ul = std::sqrt(ul);
    for (int a = 0; a < 3; ++a) u[a] = u[a] / ul;
    double v[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]};
    double R = half * std::sqrt(3.0);
    double R2 = R * 2.0;
    double* M = out->light_clip;
    auto dotc = [&](const double* a) {
        double s = a[0] * c[0];
        s = s + a[1] * c[1];
        s = s + a[2] * c[2];
        return s;
    };
    for (int a = 0; a < 3; ++a) {
        M[0 + a] = u[a] / R;
        M[4 + a] = v[a] / R;
        M[8 + a] = w[a] / R2;
        M[12 + a] = 0.0;
    }
    M[3] = -(dotc(u) / R);
    M[7] = -(dotc(v) / R);
    M[11] = 0.5 - dotc(w) / R2;
    M[15] = 1.0;
    out->shadow_bias = vs / R;
    for (int a = 0; a < 3; ++a) out->light_dir[a] = w[a];
    // FP32 affine map voxel index -> light clip (centre of voxel (0,0,0) plus one-voxel steps)
    double hv = vs * 0.5;
    double c0[3] = {out->origin[0] + hv, out->origin[1] + hv, out->origin[2] + hv};
    for (int r = 0; r < 3; ++r) {
        out->light_vox[4 * r] = float(mrow(M + 4 * r, c0[0], c0[1], c0[2]));
        for (int a = 0; a < 3; ++a) out->light_vox[4 * r + 1 + a] = float(M[4 * r + a] * vs);
    }
    out->shadow_bias_f = float(out->shadow_bias);
    return 0;
}

int orc_raster(const double M[16], uint32_t W, uint32_t H, const float* tri, uint64_t ntris, uint64_t* keys,
               int nthreads) {
    if (!M || !tri || !keys || W == 0 || H == 0) return -1;
    std::fill(keys, keys + uint64_t(W) * H, ~uint64_t(0));
    // snap every triangle once, then rasterize row slabs in parallel
    std::vector<uint32_t> owner;
    std::vector<SnapTri> all;
    float mf[16];
    for (int i = 0; i < 16; ++i) mf[i] = float(M[i]);
    for (uint64_t t = 0; t < ntris; ++t) {
        const float* p = tri + t * 9;
        bool finite = true;  // triangles with a NaN or infinite coordinate are skipped
        for (int i = 0; i < 9; ++i) finite = finite && std::isfinite(p[i]);
        if (!finite) continue;
        V4f cf[3];
        bool inside = true;
        for (int v = 0; v < 3; ++v) {
            const float x = p[v * 3], y = p[v * 3 + 1], z = p[v * 3 + 2];
            cf[v] = {frow(mf, x, y, z), frow(mf + 4, x, y, z), frow(mf + 8, x, y, z), frow(mf + 12, x, y, z)};
            inside = inside && inside_f(cf[v]);
        }
        if (inside) {
            SnapTri s;
            if (snap_tri_f(cf, W, H, s)) {
                all.push_back(s);
                owner.push_back(uint32_t(t));
            }
            continue;
        }
        V4 poly[12];
        for (int v = 0; v < 3; ++v) {
            double x = p[v * 3], y = p[v * 3 + 1], z = p[v * 3 + 2];
            poly[v] = {mrow(M, x, y, z), mrow(M + 4, x, y, z), mrow(M + 8, x, y, z), mrow(M + 12, x, y, z)};
        }
        const int n = clip_polygon(poly, 3);
        for (int i = 1; i + 1 < n; ++i) {
            SnapTri s;
            if (snap_tri(poly[0], poly[i], poly[i + 1], W, H, s)) {
                all.push_back(s);
                owner.push_back(uint32_t(t));
            }
        }
    }
    parallel_for(0, int64_t(H), nthreads, [&](int64_t rb, int64_t re) {
        for (size_t i = 0; i < all.size(); ++i) raster_tri(all[i], owner[i], W, rb, re, keys);
    });
    return 0;
}

int orc_gbuffer_resolve(const uint64_t* keys, uint32_t W, uint32_t H, const float* tri, const float* rough,
                        const float view[16], float* depth, uint32_t* normal, uint16_t* rough_out,
                        uint32_t* tri_out) {
    if (!keys || !tri || !rough || !view || !depth || !normal || !rough_out) return -1;
    double V[16], IV[16];
    for (int i = 0; i < 16; ++i) V[i] = view[i];
    if (!inverse4(V, IV)) return -1;
    Vec3<double> eye{IV[3], IV[7], IV[11]};
    for (uint64_t i = 0; i < uint64_t(W) * H; ++i) {
        uint64_t k = keys[i];
        if (k == ~uint64_t(0)) {
            depth[i] = 1.0f;
            normal[i] = 0;
            rough_out[i] = 0;
            if (tri_out) tri_out[i] = 0xffffffffu;
            continue;
        }
        uint32_t t = uint32_t(k & 0xffffffffu);
        depth[i] = bits_float(uint32_t(k >> 32));
        const float* p = tri + uint64_t(t) * 9;
        Vec3<double> p0{p[0], p[1], p[2]}, p1{p[3], p[4], p[5]}, p2{p[6], p[7], p[8]};
        Vec3<double> n = vnorm(vcross(vsub(p1, p0), vsub(p2, p0)));
        if (vdot(n, vsub(eye, p0)) < 0.0) n = vmul(n, -1.0);
        Vec3<double> nv = vnorm(Vec3<double>{V[0] * n.x + V[1] * n.y + V[2] * n.z, V[4] * n.x + V[5] * n.y + V[6] * n.z,
                                             V[8] * n.x + V[9] * n.y + V[10] * n.z});
        normal[i] = oct_encode_d(nv);
        rough_out[i] = f2h(double(rough[t]));
        if (tri_out) tri_out[i] = t;
    }
    return 0;
}

int orc_voxelize_f64(const f184gi_grid_frame* frame, uint32_t dim, uint32_t res, const float* tri,
                     const uint32_t* albedo, uint64_t ntris, const f184gi_light* light, const float* shadow,
                     double* rgba, uint32_t* counts, int nthreads) {
    return voxelize_impl<double>(frame, dim, res, tri, albedo, ntris, light, shadow, rgba, counts, nthreads);
}
int orc_voxelize_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t res, const float* tri,
                     const uint32_t* albedo, uint64_t ntris, const f184gi_light* light, const float* shadow,
                     float* rgba, uint32_t* counts, int nthreads) {
    return voxelize_impl<float>(frame, dim, res, tri, albedo, ntris, light, shadow, rgba, counts, nthreads);
}

int orc_shade(const f184gi_grid_frame* frame, uint32_t res, const float* shadow, const uint32_t* ijk, uint64_t n,
              uint8_t* lit) {
    if (!frame || !shadow || !ijk || !lit) return -1;
    for (uint64_t i = 0; i < n; ++i)
        lit[i] = shade_voxel(*frame, res, shadow, ijk[i * 3], ijk[i * 3 + 1], ijk[i * 3 + 2]) ? 1 : 0;
    return 0;
}

int orc_mip_f64(double* chain, uint32_t dim, uint32_t levels, int nthreads) {
    return mip_impl(chain, dim, levels, nthreads);
}
int orc_mip_f32(float* chain, uint32_t dim, uint32_t levels, int nthreads) {
    return mip_impl(chain, dim, levels, nthreads);
}
int orc_mip_aniso_f64(double* chain, uint32_t dim, uint32_t levels, int nthreads) {
    return mip_aniso_impl(chain, dim, levels, nthreads);
}

int orc_trace_f64(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso,
                  const double* chain, const float view[16], const float proj[16], uint32_t W, uint32_t H,
                  const float* depth, const uint32_t* normal, const uint16_t* rough,
                  const f184gi_cone_params* params, double* out, uint32_t rb, uint32_t re, int nthreads) {
    return trace_impl<double>(frame, dim, levels, aniso, chain, view, proj, W, H, depth, normal, rough, params,
                              out, rb, re, nthreads);
}
int orc_trace_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso,
                  const float* chain, const float view[16], const float proj[16], uint32_t W, uint32_t H,
                  const float* depth, const uint32_t* normal, const uint16_t* rough,
                  const f184gi_cone_params* params, float* out, uint32_t rb, uint32_t re, int nthreads) {
    return trace_impl<float>(frame, dim, levels, aniso, chain, view, proj, W, H, depth, normal, rough, params,
                             out, rb, re, nthreads);
}

int orc_trace_count_f32(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso,
                        const float* chain, const float view[16], const float proj[16], uint32_t W, uint32_t H,
                        const float* depth, const uint32_t* normal, const uint16_t* rough,
                        const f184gi_cone_params* params, float* out, uint32_t rb, uint32_t re, int nthreads,
                        uint64_t counts[2]) {
    if (!counts) return -1;
    counts[0] = counts[1] = 0;
    return trace_impl<float>(frame, dim, levels, aniso, chain, view, proj, W, H, depth, normal, rough, params, out,
                             rb, re, nthreads, counts);
}

int orc_cone_f64(const double* chain, uint32_t dim, uint32_t levels, uint32_t aniso, const double o[3],
                 const double dir[3], double tan_half, const f184gi_cone_params* params, double out[4]) {
    if (!chain || !o || !dir || !out) return -1;
    f184gi_cone_params p = params ? *params : default_params();
    Chain<double> ch = make_chain(chain, dim, levels, aniso != 0);
    double tmax = p.max_distance > 0 ? double(p.max_distance) : double(dim) * std::sqrt(3.0);
    cone(ch, Vec3<double>{o[0], o[1], o[2]}, Vec3<double>{dir[0], dir[1], dir[2]}, tan_half, p, tmax, out);
    return 0;
}

void orc_make_coord_space(const double n[3], double out[9]) {
    Vec3<double> x, y, z;
    make_coord_space(Vec3<double>{n[0], n[1], n[2]}, x, y, z);
    const Vec3<double> c[3] = {x, y, z};
    for (int i = 0; i < 3; ++i) {
        out[i * 3 + 0] = c[i].x;
        out[i * 3 + 1] = c[i].y;
        out[i * 3 + 2] = c[i].z;
    }
}

// main.lua:269: uint(BaseColor.r * 31) << 11 | uint(BaseColor.g * 63) << 5 | uint(BaseColor.b * 31)
uint32_t orc_pack_color565(const float rgb[3]) {
    return (uint32_t(rgb[0] * 31.0f) << 11) | (uint32_t(rgb[1] * 63.0f) << 5) | uint32_t(rgb[2] * 31.0f);
}
// main.lua:270: uint(n.r * 16 + 15) << 11 | uint(n.g * 32 + 31) << 5 | uint(n.b * 16 + 15)
uint32_t orc_pack_normal565(const float n[3]) {
    return (uint32_t(n[0] * 16.0f + 15.0f) << 11) | (uint32_t(n[1] * 32.0f + 31.0f) << 5) |
           uint32_t(n[2] * 16.0f + 15.0f);
}
void orc_unpack_color565(uint32_t x, double out[3]) {
    out[0] = double((x & 0xF800u) >> 11) / 31.0;
    out[1] = double((x & 0x7E0u) >> 5) / 63.0;
    out[2] = double(x & 0x1Fu) / 31.0;
}
// indirect.frag:96-102 reads the channels in the opposite order from the pack (x from the low bits)
void orc_unpack_normal565(uint32_t x, double out[3]) {
    Vec3<double> v{double(x & 0x1Fu) / 16.0 - 1.0, double((x & 0x7E0u) >> 5) / 32.0 - 1.0,
                   double((x & 0xF800u) >> 11) / 16.0 - 1.0};
    v = vnorm(v);
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}
int orc_dominant_axis(const float v0[3], const float v1[3], const float v2[3]) {
    float a[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    float b[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    float n[3] = {std::fabs(a[1] * b[2] - a[2] * b[1]), std::fabs(a[2] * b[0] - a[0] * b[2]),
                  std::fabs(a[0] * b[1] - a[1] * b[0])};
    if (n[0] > n[1]) return n[0] > n[2] ? 1 : 0;
    return n[1] > n[2] ? 2 : 0;
}
void orc_hemisphere_sample_cos(double u, double v, double out[3]) {
    const double PI = 3.1415926;  // math.inc:1 uses this truncated constant
    double phi = v * 2.0 * PI;
    double ct = std::sqrt(1.0 - u);
    double st = std::sqrt(1.0 - ct * ct);
    out[0] = std::cos(phi) * st;
    out[1] = std::sin(phi) * st;
    out[2] = ct;
}
uint32_t orc_oct_encode(const double n[3]) { return oct_encode_d(vnorm(Vec3<double>{n[0], n[1], n[2]})); }
void orc_oct_decode(uint32_t packed, double out[3]) {
    Vec3<double> v = oct_decode<double>(packed);
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}
uint16_t orc_float_to_half(double x) { return f2h(x); }
double orc_half_to_float(uint16_t h) { return h2f(h); }

}  // extern "C"

// ---------------- reference-faithful volume and march ----------------
//
// The reference's own voxelization (Pipelang/Internal/main.lua:83-144 VoxelGS, :242-275 VoxelPS: dominant-axis
// raster at pixel centres, 565 packing) and its single-ray march with a second bounce
// (Shader/Lighting/indirect.frag:104-222 without the temporal blend).  The FP32 march below is the device's
// operation sequence (each operation rounded on its own, integer hash for the reference's noise, a Taylor sin/cos
// of the sample angle), so it agrees bit for bit; the FP64 march is the same method in double with std::sin/cos
// and std::pow.

namespace {

struct RefMaps32 {
    float s, b[3], w2l[12];
};
RefMaps32 ref_maps(const f184gi_grid_frame* fr) {
    RefMaps32 m;
    const double inv = fr->inv_voxel_fixed * (1.0 / 256.0);
    m.s = float(inv);
    for (int a = 0; a < 3; ++a) m.b[a] = float(-fr->origin[a] * inv);
    for (int k = 0; k < 12; ++k) m.w2l[k] = float(fr->light_clip[k]);
    return m;
}

template <class T>
struct RefMaps {
    T s, b[3], w2l[12];
};
template <class T>
RefMaps<T> ref_maps_t(const f184gi_grid_frame* fr) {
    RefMaps<T> m;
    if (std::is_same<T, float>::value) {
        RefMaps32 f = ref_maps(fr);
        m.s = T(f.s);
        for (int a = 0; a < 3; ++a) m.b[a] = T(f.b[a]);
        for (int k = 0; k < 12; ++k) m.w2l[k] = T(f.w2l[k]);
    } else {
        const double inv = fr->inv_voxel_fixed * (1.0 / 256.0);
        m.s = T(inv);
        for (int a = 0; a < 3; ++a) m.b[a] = T(-fr->origin[a] * inv);
        for (int k = 0; k < 12; ++k) m.w2l[k] = T(fr->light_clip[k]);
    }
    return m;
}

inline uint32_t lowbias32(uint32_t x) {  // C. Wellons' integer hash
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// sin, cos of 2 pi v (v in [0, 1)) as the device evaluates them: quadrant, exact remainder in turns, Taylor series
void sincos_turns32(float v, float& s, float& c) {
    const int q = int(std::floor(v * 4.0f + 0.5f));
    const float r = v - float(q) * 0.25f;
    const float x = r * 6.28318530717958647692f;
    const float x2 = x * x;
    float ps = -1.0f / 5040.0f + x2 * (1.0f / 362880.0f);
    ps = 1.0f / 120.0f + x2 * ps;
    ps = -1.0f / 6.0f + x2 * ps;
    ps = 1.0f + x2 * ps;
    const float sn = x * ps;
    float pc = 1.0f / 40320.0f + x2 * (-1.0f / 3628800.0f);
    pc = -1.0f / 720.0f + x2 * pc;
    pc = 1.0f / 24.0f + x2 * pc;
    pc = -0.5f + x2 * pc;
    const float cs = 1.0f + x2 * pc;
    switch (q & 3) {
        case 0: s = sn, c = cs; break;
        case 1: s = cs, c = -sn; break;
        case 2: s = -sn, c = -cs; break;
        default: s = -cs, c = sn; break;
    }
}

template <class T>
Vec3<T> rnorm(Vec3<T> v) {  // v / length(v), zero stays zero
    T l = std::sqrt(vdot(v, v));
    return l > T(0) ? Vec3<T>{v.x / l, v.y / l, v.z / l} : v;
}
template <class T>
Vec3<T> rcross(Vec3<T> a, Vec3<T> b) {
    return Vec3<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

template <class T>
struct RefHit {
    Vec3<T> wpos, wnorm, brdf;
    bool hit;
};

template <class T>
struct MarchCtx {
    RefMaps<T> m;
    const uint32_t* vol;
    uint32_t dim, res;
    const float* shadow;  // FP32 depth, 1.0 where empty
    T lum[3], ldir[3];
    T pow5[32], pow6[64];
    f184gi_march_params p;
};

template <class T>
Vec3<T> ref_w2v(const RefMaps<T>& m, Vec3<T> p) {
    return Vec3<T>{p.x * m.s + m.b[0], p.y * m.s + m.b[1], p.z * m.s + m.b[2]};
}

// The two uniform numbers of ray `seed` of pixel `pix` in frame `frame`: they stand where indirect.frag:113-117
// draws rands.x (the cosine-sampling u) and rands.y (the angle v, also the start offset) from its frame-dependent noise.
inline void march_rands(uint32_t frame, uint32_t pix, uint32_t seed, float& ru, float& rv) {
    const uint32_t key = lowbias32(frame * 16u + seed * 2u);
    ru = float(lowbias32(pix ^ key) >> 8) * 5.9604644775390625e-8f;
    rv = float(lowbias32(pix ^ (key + 0x9e3779b9u)) >> 8) * 5.9604644775390625e-8f;
}

template <class T>
Vec3<T> march_ray(const MarchCtx<T>& C, uint32_t pix, Vec3<T> wpos, Vec3<T> wnorm, uint32_t seed, RefHit<T>& hit) {
    hit.hit = false;
    Vec3<T> lo{T(0), T(0), T(0)};
    float ru, rv;
    march_rands(C.p.frame, pix, seed, ru, rv);
    const T ct = std::sqrt(T(1) - T(ru));
    const T st = std::sqrt(T(1) - ct * ct);
    T sp, cp;
    if (std::is_same<T, float>::value) {
        float s32, c32;
        sincos_turns32(rv, s32, c32);
        sp = T(s32), cp = T(c32);
    } else {
        const double ang = double(rv) * 6.283185307179586476925;
        sp = T(std::sin(ang)), cp = T(std::cos(ang));
    }
    const Vec3<T> dl{cp * st, sp * st, ct};
    // make_coord_space (indirect.frag:71-86)
    Vec3<T> h = wnorm;
    {
        const T ax = std::fabs(h.x), ay = std::fabs(h.y), az = std::fabs(h.z);
        if (ax <= ay && ax <= az) h.x = T(1);
        else if (ay <= ax && ay <= az) h.y = T(1);
        else h.z = T(1);
    }
    const Vec3<T> bz = rnorm(wnorm);
    const Vec3<T> by = rnorm(rcross(h, bz));
    const Vec3<T> bx = rnorm(rcross(bz, by));
    Vec3<T> dir{(bx.x * dl.x + by.x * dl.y) + bz.x * dl.z, (bx.y * dl.x + by.y * dl.y) + bz.y * dl.z,
                (bx.z * dl.x + by.z * dl.y) + bz.z * dl.z};
    if (vdot(dir, wnorm) < T(0)) dir = Vec3<T>{-dir.x, -dir.y, -dir.z};
    const T ndd = vdot(dir, wnorm);
    const T step = T(C.p.step_size);
    const T so = T(1) + T(rv);
    Vec3<T> mp{wpos.x + ((dir.x * so) * step) / ndd, wpos.y + ((dir.y * so) * step) / ndd,
               wpos.z + ((dir.z * so) * step) / ndd};
    const Vec3<T> sv = ref_w2v(C.m, wpos);
    int px = int(sv.x), py = int(sv.y), pz = int(sv.z);
    const T maxd = T(C.dim - 1);
    uint32_t i = 0;
    for (; i < C.p.max_steps; ++i) {
        mp = Vec3<T>{mp.x + dir.x * step, mp.y + dir.y * step, mp.z + dir.z * step};
        const Vec3<T> vp = ref_w2v(C.m, mp);
        if (vp.x < T(0) || vp.y < T(0) || vp.z < T(0) || vp.x > maxd || vp.y > maxd || vp.z > maxd) break;
        const int ix = int(vp.x), iy = int(vp.y), iz = int(vp.z);
        if (ix == px && iy == py && iz == pz) continue;
        const uint32_t data = C.vol[(uint64_t(iz) * C.dim + uint64_t(iy)) * C.dim + uint64_t(ix)];
        px = ix, py = iy, pz = iz;
        const uint32_t r = data & 0xffffu, g = data >> 16;
        if (r == 0) continue;
        const Vec3<T> col{C.pow5[(r >> 11) & 31u], C.pow6[(r >> 5) & 63u], C.pow5[r & 31u]};
        const Vec3<T> vn = rnorm(Vec3<T>{T(g & 0x1fu) / T(16) - T(1), T((g >> 5) & 0x3fu) / T(32) - T(1),
                                         T((g >> 11) & 0x1fu) / T(16) - T(1)});
        const T no = T(C.p.normal_offset);
        const Vec3<T> q{mp.x + vn.x * no, mp.y + vn.y * no, mp.z + vn.z * no};
        const T* L = C.m.w2l;
        const T lx = ((L[0] * q.x + L[1] * q.y) + L[2] * q.z) + L[3];
        const T ly = ((L[4] * q.x + L[5] * q.y) + L[6] * q.z) + L[7];
        const T lz = ((L[8] * q.x + L[9] * q.y) + L[10] * q.z) + L[11];
        const int tx = int((lx * T(0.5) + T(0.5)) * T(C.res));
        const int ty = int((ly * T(0.5) + T(0.5)) * T(C.res));
        T shade = T(1);
        if (unsigned(tx) < C.res && unsigned(ty) < C.res) {
            const T sd = T(C.shadow[uint64_t(ty) * C.res + uint64_t(tx)]);
            shade = sd < lz + T(C.p.shadow_bias) ? T(0) : T(1);
        }
        const T lam = std::fabs(vdot(Vec3<T>{-C.ldir[0], -C.ldir[1], -C.ldir[2]}, vn));
        const T den = std::max(T(0.01f), ndd);
        const Vec3<T> br{(lam * col.x) / den, (lam * col.y) / den, (lam * col.z) / den};
        hit.brdf = br;
        lo = Vec3<T>{lo.x + (C.lum[0] * shade) * br.x, lo.y + (C.lum[1] * shade) * br.y,
                     lo.z + (C.lum[2] * shade) * br.z};
        hit.wpos = mp;
        hit.wnorm = vn;
        hit.hit = true;
        break;
    }
    if (!hit.hit && i == C.p.max_steps) {
        const T den = std::max(T(0.01f), ndd);
        T t = ndd / T(0.01f);
        t = std::min(std::max(t, T(0)), T(1));
        const T ss = (t * t) * (T(3) - T(2) * t);
        const T sc = T(C.p.sky_scale);
        lo = Vec3<T>{lo.x + ((T(C.p.sky[0]) * sc) / den) * ss, lo.y + ((T(C.p.sky[1]) * sc) / den) * ss,
                     lo.z + ((T(C.p.sky[2]) * sc) / den) * ss};
    }
    return lo;
}

template <class T>
MarchCtx<T> march_ctx(const f184gi_grid_frame* frame, uint32_t dim, const uint32_t* vol, const float* shadow,
                      uint32_t res, const f184gi_light* light, const f184gi_march_params* params) {
    MarchCtx<T> C;
    C.m = ref_maps_t<T>(frame);
    C.vol = vol;
    C.dim = dim;
    C.res = res;
    C.shadow = shadow;
    C.p = *params;
    for (int a = 0; a < 3; ++a) C.lum[a] = T(light->luminance[a]), C.ldir[a] = T(light->direction[a]);
    for (int k = 0; k < 32; ++k)
        C.pow5[k] = std::is_same<T, float>::value ? T(float(std::pow(double(float(k) / 31.0f), 2.2)))
                                                  : T(std::pow(double(k) / 31.0, 2.2));
    for (int k = 0; k < 64; ++k)
        C.pow6[k] = std::is_same<T, float>::value ? T(float(std::pow(double(float(k) / 63.0f), 2.2)))
                                                  : T(std::pow(double(k) / 63.0, 2.2));
    return C;
}

// One pixel of the reference's combine (indirect.frag:197-222 without the temporal blend): `rays` rays, each with
// its second bounce weighted by the first hit's brdf, times 1 / rays.
template <class T>
Vec3<T> march_pixel(const MarchCtx<T>& C, uint32_t pix, Vec3<T> wpos, Vec3<T> wn) {
    Vec3<T> acc{T(0), T(0), T(0)};
    RefHit<T> h;
    for (uint32_t k = 0; k < C.p.rays; ++k) {
        const Vec3<T> l1 = march_ray(C, pix, wpos, wn, 2 * k, h);
        acc = Vec3<T>{acc.x + l1.x, acc.y + l1.y, acc.z + l1.z};
        if (h.hit && C.p.second_bounce) {
            const Vec3<T> br = h.brdf;
            RefHit<T> h2;
            const Vec3<T> l2 = march_ray(C, pix, h.wpos, h.wnorm, 2 * k + 1, h2);
            acc = Vec3<T>{acc.x + br.x * l2.x, acc.y + br.y * l2.y, acc.z + br.z * l2.z};
        }
    }
    const T sc = T(1) / T(float(C.p.rays));
    return Vec3<T>{acc.x * sc, acc.y * sc, acc.z * sc};
}

template <class T>
int march_impl(const f184gi_grid_frame* frame, uint32_t dim, const uint32_t* vol, const float* shadow, uint32_t res,
               const f184gi_light* light, const float view[16], const float proj[16], uint32_t W, uint32_t H,
               const float* depth, const uint32_t* normal, const f184gi_march_params* params, T* out,
               uint32_t row_begin, uint32_t row_end, int nthreads) {
    if (!frame || !vol || !shadow || !light || !view || !proj || !depth || !normal || !params || !out) return -1;
    const MarchCtx<T> C = march_ctx<T>(frame, dim, vol, shadow, res, light, params);
    double V[16], P[16], IV[16], IP[16];
    for (int i = 0; i < 16; ++i) V[i] = view[i], P[i] = proj[i];
    if (!inverse4(V, IV) || !inverse4(P, IP)) return -1;
    float iv[16], ip[16];
    for (int i = 0; i < 16; ++i) iv[i] = float(IV[i]), ip[i] = float(IP[i]);
    const int64_t p_begin = int64_t(row_begin) * W, p_end = int64_t(std::min(row_end, H)) * W;
    parallel_for(p_begin, p_end, nthreads, [&](int64_t pb, int64_t pe) {
        for (int64_t pix = pb; pix < pe; ++pix) {
            const uint32_t px = uint32_t(pix % W), py = uint32_t(pix / W);
            T* o = out + uint64_t(pix) * 4;
            const float d = depth[pix];
            if (!(d < 1.0f)) {
                o[0] = o[1] = o[2] = o[3] = T(0);
                continue;
            }
            Vec3<T> cs, wpos, wn;
            if (std::is_same<T, float>::value) {  // the device's sequence
                const float nx = ((float(px) + 0.5f) / float(W)) * 2.0f - 1.0f;
                const float ny = ((float(py) + 0.5f) / float(H)) * 2.0f - 1.0f;
                const float vx = ((ip[0] * nx + ip[1] * ny) + ip[2] * d) + ip[3];
                const float vy = ((ip[4] * nx + ip[5] * ny) + ip[6] * d) + ip[7];
                const double vz = ((IP[8] * double(nx) + IP[9] * double(ny)) + IP[10] * double(d)) + IP[11];
                const double vw = ((IP[12] * double(nx) + IP[13] * double(ny)) + IP[14] * double(d)) + IP[15];
                const double rw = 1.0 / vw;
                const float rwf = float(rw);
                const Vec3<float> c{vx * rwf, vy * rwf, float(vz * rw)};
                const Vec3<float> w{((iv[0] * c.x + iv[1] * c.y) + iv[2] * c.z) + iv[3],
                                    ((iv[4] * c.x + iv[5] * c.y) + iv[6] * c.z) + iv[7],
                                    ((iv[8] * c.x + iv[9] * c.y) + iv[10] * c.z) + iv[11]};
                const uint32_t pn = normal[pix];
                Vec3<float> on{float(h2f(uint16_t(pn & 0xffffu))), float(h2f(uint16_t(pn >> 16))), 0.0f};
                on.z = (1.0f - std::fabs(on.x)) - std::fabs(on.y);
                if (on.z < 0.0f) {
                    const float ox = on.x, oy = on.y;
                    on.x = (1.0f - std::fabs(oy)) * (ox >= 0.0f ? 1.0f : -1.0f);
                    on.y = (1.0f - std::fabs(ox)) * (oy >= 0.0f ? 1.0f : -1.0f);
                }
                const Vec3<float> cn = rnorm(on);
                const Vec3<float> n{(iv[0] * cn.x + iv[1] * cn.y) + iv[2] * cn.z, (iv[4] * cn.x + iv[5] * cn.y) + iv[6] * cn.z,
                                    (iv[8] * cn.x + iv[9] * cn.y) + iv[10] * cn.z};
                cs = Vec3<T>{T(c.x), T(c.y), T(c.z)};
                wpos = Vec3<T>{T(w.x), T(w.y), T(w.z)};
                wn = Vec3<T>{T(n.x), T(n.y), T(n.z)};
            } else {
                const double nx = (double(px) + 0.5) / double(W) * 2.0 - 1.0;
                const double ny = (double(py) + 0.5) / double(H) * 2.0 - 1.0;
                double vp[4];
                for (int r = 0; r < 4; ++r) vp[r] = IP[r * 4] * nx + IP[r * 4 + 1] * ny + IP[r * 4 + 2] * double(d) + IP[r * 4 + 3];
                const Vec3<double> c{vp[0] / vp[3], vp[1] / vp[3], vp[2] / vp[3]};
                const Vec3<double> cn = oct_decode<double>(normal[pix]);
                cs = Vec3<T>{T(c.x), T(c.y), T(c.z)};
                wpos = Vec3<T>{T(IV[0] * c.x + IV[1] * c.y + IV[2] * c.z + IV[3]),
                               T(IV[4] * c.x + IV[5] * c.y + IV[6] * c.z + IV[7]),
                               T(IV[8] * c.x + IV[9] * c.y + IV[10] * c.z + IV[11])};
                wn = Vec3<T>{T(IV[0] * cn.x + IV[1] * cn.y + IV[2] * cn.z), T(IV[4] * cn.x + IV[5] * cn.y + IV[6] * cn.z),
                             T(IV[8] * cn.x + IV[9] * cn.y + IV[10] * cn.z)};
            }
            const Vec3<T> acc = march_pixel(C, uint32_t(pix), wpos, wn);
            o[0] = acc.x, o[1] = acc.y, o[2] = acc.z, o[3] = -cs.z;
        }
    });
    return 0;
}

// The reference volume: dominant-axis raster at pixel centres (edge ties: dy > 0, or dy == 0 and dx < 0), the
// VoxelPS swizzles, highest triangle index wins, 565 packing of albedo and face normal.
int refvox_impl(const f184gi_grid_frame* fr, uint32_t dim, const float* tri, const uint32_t* albedo, uint64_t ntris,
                uint32_t* vol) {
    const RefMaps32 m = ref_maps(fr);
    const uint64_t nvox = uint64_t(dim) * dim * dim;
    std::vector<uint32_t> owner(nvox, 0);
    const float fd = float(dim), inv_dim = 1.0f / fd, maxd = float(dim - 1);
    for (uint64_t t = 0; t < ntris; ++t) {
        float u[3][3];
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a) u[v][a] = tri[t * 9 + 3 * v + a] * m.s + m.b[a];
        const float e1[3] = {u[1][0] - u[0][0], u[1][1] - u[0][1], u[1][2] - u[0][2]};
        const float e2[3] = {u[2][0] - u[0][0], u[2][1] - u[0][1], u[2][2] - u[0][2]};
        const float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const float ax = std::fabs(n[0]), ay = std::fabs(n[1]), az = std::fabs(n[2]);
        const int o = ax > ay ? (ax > az ? 1 : 0) : (ay > az ? 2 : 0);
        float sx[3], sy[3], sz[3];
        bool ok = true;
        for (int v = 0; v < 3; ++v) {
            if (o == 0) sx[v] = u[v][0], sy[v] = u[v][1], sz[v] = u[v][2] * inv_dim;
            else if (o == 1) sx[v] = u[v][2], sy[v] = u[v][1], sz[v] = 1.0f - u[v][0] * inv_dim;
            else sx[v] = u[v][0], sy[v] = fd - u[v][2], sz[v] = u[v][1] * inv_dim;
            ok = ok && std::fabs(sx[v]) < 4096.0f && std::fabs(sy[v]) < 4096.0f;
        }
        if (!ok) continue;
        int32_t X[3], Y[3];
        for (int v = 0; v < 3; ++v) X[v] = int32_t(std::nearbyint(sx[v] * 256.0f)), Y[v] = int32_t(std::nearbyint(sy[v] * 256.0f));
        int64_t det = int64_t(X[1] - X[0]) * (Y[2] - Y[0]) - int64_t(X[2] - X[0]) * (Y[1] - Y[0]);
        if (det == 0) continue;
        int i1 = 1, i2 = 2;
        if (det < 0) i1 = 2, i2 = 1, det = -det;
        const int id[3] = {0, i1, i2};
        int32_t RX[3], RY[3];
        for (int v = 0; v < 3; ++v) RX[v] = X[id[v]], RY[v] = Y[id[v]];
        const double z0 = sz[0], z1 = sz[i1], z2 = sz[i2];
        const double dx1 = RX[1] - RX[0], dy1 = RY[1] - RY[0], dx2 = RX[2] - RX[0], dy2 = RY[2] - RY[0];
        const double dz1 = z1 - z0, dz2 = z2 - z0;
        const float fz0 = float(z0);
        const float fa_ = float((dz1 * dy2 - dz2 * dy1) / double(det));
        const float fb_ = float((dz2 * dx1 - dz1 * dx2) / double(det));
        const int32_t mnx = std::min(RX[0], std::min(RX[1], RX[2])), mxx = std::max(RX[0], std::max(RX[1], RX[2]));
        const int32_t mny = std::min(RY[0], std::min(RY[1], RY[2])), mxy = std::max(RY[0], std::max(RY[1], RY[2]));
        const int32_t x0 = std::max(0, (mnx - 128 + 255) >> 8), x1 = std::min(int32_t(dim) - 1, (mxx - 128) >> 8);
        const int32_t y0 = std::max(0, (mny - 128 + 255) >> 8), y1 = std::min(int32_t(dim) - 1, (mxy - 128) >> 8);
        int64_t ex[3], ey[3];
        bool incl[3];
        for (int e = 0; e < 3; ++e) {
            const int nn = (e + 1) % 3;
            ex[e] = int64_t(RX[nn]) - RX[e];
            ey[e] = int64_t(RY[nn]) - RY[e];
            incl[e] = ey[e] > 0 || (ey[e] == 0 && ex[e] < 0);
        }
        for (int32_t py = y0; py <= y1; ++py)
            for (int32_t px = x0; px <= x1; ++px) {
                const int64_t cx = int64_t(px) * 256 + 128, cy = int64_t(py) * 256 + 128;
                bool in = true;
                for (int e = 0; e < 3; ++e) {
                    const int64_t w = ex[e] * (cy - RY[e]) - ey[e] * (cx - RX[e]);
                    in = in && (w > 0 || (w == 0 && incl[e]));
                }
                if (!in) continue;
                const float z = (fz0 + fa_ * float(cx - RX[0])) + fb_ * float(cy - RY[0]);
                int vx, vy, vz;
                if (o == 0) vx = px, vy = py, vz = int(z * maxd);
                else if (o == 1) vx = int((1.0f - z) * maxd), vy = py, vz = px;
                else vx = px, vy = int(z * maxd), vz = int(maxd - (float(py) + 0.5f));
                if (unsigned(vx) >= dim || unsigned(vy) >= dim || unsigned(vz) >= dim) continue;
                uint32_t& ow = owner[(uint64_t(vz) * dim + uint64_t(vy)) * dim + uint64_t(vx)];
                ow = std::max(ow, uint32_t(t + 1));
            }
    }
    for (uint64_t v = 0; v < nvox; ++v) {
        const uint32_t o = owner[v];
        if (!o) {
            vol[v] = 0;
            continue;
        }
        const uint64_t t = o - 1;
        const uint32_t al = albedo[t];
        const float cr = float(al & 255u) / 255.0f, cg = float((al >> 8) & 255u) / 255.0f,
                    cb = float((al >> 16) & 255u) / 255.0f;
        const uint32_t color = (uint32_t(cr * 31.0f) << 11) | (uint32_t(cg * 63.0f) << 5) | uint32_t(cb * 31.0f);
        const float* p = tri + t * 9;
        const Vec3<float> n = rnorm(rcross(Vec3<float>{p[3] - p[0], p[4] - p[1], p[5] - p[2]},
                                           Vec3<float>{p[6] - p[0], p[7] - p[1], p[8] - p[2]}));
        const uint32_t nx = uint32_t(std::max(0.0f, n.x * 16.0f + 15.0f));
        const uint32_t ny = uint32_t(std::max(0.0f, n.y * 32.0f + 31.0f));
        const uint32_t nz = uint32_t(std::max(0.0f, n.z * 16.0f + 15.0f));
        const uint32_t nn = ((nx << 11) | (ny << 5) | nz) & 0xffffu;
        vol[v] = (color & 0xffffu) | (nn << 16);
    }
    return 0;
}

}  // namespace

extern "C" {

int orc_refvox(const f184gi_grid_frame* frame, uint32_t dim, const float* tri, const uint32_t* albedo,
               uint64_t ntris, uint32_t* vol) {
    if (!frame || !vol || (ntris && (!tri || !albedo))) return -1;
    return refvox_impl(frame, dim, tri, albedo, ntris, vol);
}
int orc_march_f32(const f184gi_grid_frame* frame, uint32_t dim, const uint32_t* vol, const float* shadow,
                  uint32_t res, const f184gi_light* light, const float view[16], const float proj[16], uint32_t W,
                  uint32_t H, const float* depth, const uint32_t* normal, const f184gi_march_params* params,
                  float* out, uint32_t row_begin, uint32_t row_end, int nthreads) {
    return march_impl<float>(frame, dim, vol, shadow, res, light, view, proj, W, H, depth, normal, params, out,
                             row_begin, row_end, nthreads);
}
int orc_march_f64(const f184gi_grid_frame* frame, uint32_t dim, const uint32_t* vol, const float* shadow,
                  uint32_t res, const f184gi_light* light, const float view[16], const float proj[16], uint32_t W,
                  uint32_t H, const float* depth, const uint32_t* normal, const f184gi_march_params* params,
                  double* out, uint32_t row_begin, uint32_t row_end, int nthreads) {
    return march_impl<double>(frame, dim, vol, shadow, res, light, view, proj, W, H, depth, normal, params, out,
                              row_begin, row_end, nthreads);
}
void orc_sincos_turns(float v, float* s, float* c) { sincos_turns32(v, *s, *c); }

// The FP32 march of n world-space points (position, normal), pixel index pix[i] for the ray numbers: the part of
// orc_march_f32 after the G-buffer decode, for comparison with the reference's own getIndirect text.
int orc_march_points_f32(const f184gi_grid_frame* frame, uint32_t dim, const uint32_t* vol, const float* shadow,
                         uint32_t res, const f184gi_light* light, const f184gi_march_params* params,
                         const uint32_t* pix, const float* wpos, const float* wnorm, uint64_t n, float* out) {
    if (!frame || !vol || !shadow || !light || !params || !pix || !wpos || !wnorm || !out) return -1;
    const MarchCtx<float> C = march_ctx<float>(frame, dim, vol, shadow, res, light, params);
    parallel_for(0, int64_t(n), 0, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const Vec3<float> p{wpos[i * 3], wpos[i * 3 + 1], wpos[i * 3 + 2]};
            const Vec3<float> nn{wnorm[i * 3], wnorm[i * 3 + 1], wnorm[i * 3 + 2]};
            const Vec3<float> o = march_pixel(C, pix[i], p, nn);
            out[i * 3] = o.x, out[i * 3 + 1] = o.y, out[i * 3 + 2] = o.z;
        }
    });
    return 0;
}

// rands[i][seed][0..1] = (u, v) of ray `seed` (0 .. 2 * rays - 1) of pixel pix[i]
void orc_march_rands(uint32_t frame, const uint32_t* pix, uint64_t n, uint32_t seeds, float* rands) {
    for (uint64_t i = 0; i < n; ++i)
        for (uint32_t k = 0; k < seeds; ++k) march_rands(frame, pix[i], k, rands[(i * seeds + k) * 2], rands[(i * seeds + k) * 2 + 1]);
}

}  // extern "C"

// ---------------- depth-aware blur (Shader/Lighting/bilateralBlur.inc:19-73) ----------------

namespace {

float exp2_poly32(float t) {  // the device's exp2: 2^round(t) times a degree-7 Taylor polynomial
    if (!(t > -126.0f)) return 0.0f;
    t = std::min(t, 127.0f);
    const int n = int(std::nearbyint(t));
    const float x = (t - float(n)) * 0.693147180559945309f;
    float p = 1.0f / 720.0f + x * (1.0f / 5040.0f);
    p = 1.0f / 120.0f + x * p;
    p = 1.0f / 24.0f + x * p;
    p = 1.0f / 6.0f + x * p;
    p = 0.5f + x * p;
    p = 1.0f + x * p;
    p = 1.0f + x * p;
    const uint32_t bits = uint32_t(n + 127) << 23;
    float scale;
    std::memcpy(&scale, &bits, 4);
    return p * scale;
}

template <class T>
T blur_weight(T r, T d, T d0) {
    const T dz = (d0 - d) * T(512);
    const T t = ((-r * r) * (T(1) / T(32))) - dz * dz;
    if (std::is_same<T, float>::value) return T(exp2_poly32(float(t)));
    return T(std::exp2(double(t)));
}

template <class T>
void blur_pass_impl(const T* in, const float* depth, uint32_t W, uint32_t H, int axis, T* out) {
    const int n = axis ? int(W) : int(H);
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            const int c = axis ? int(x) : int(y);
            auto at = [&](int k) -> uint64_t {
                k = k < 0 ? 0 : (k >= n ? n - 1 : k);
                return axis ? uint64_t(y) * W + uint64_t(k) : uint64_t(k) * W + x;
            };
            const uint64_t p0 = uint64_t(y) * W + x;
            const T z0 = T(depth[p0]);
            T tr = in[p0 * 4], tg = in[p0 * 4 + 1], tb = in[p0 * 4 + 2], tw = T(1);
            auto tap = [&](int off, T r) {
                const uint64_t q = at(c + off);
                const T w = blur_weight<T>(r, T(depth[q]), z0);
                tr = tr + in[q * 4] * w;
                tg = tg + in[q * 4 + 1] * w;
                tb = tb + in[q * 4 + 2] * w;
                tw = tw + w;
            };
            for (int i = 1; i <= 4; ++i) {
                tap(2 * i, T(i));
                tap(-2 * i, T(i));
            }
            for (int i = 5; i <= 7; i += 2) {
                tap(2 * i + 1, T(i));
                tap(-2 * i - 1, T(i));
            }
            out[p0 * 4] = tr / tw, out[p0 * 4 + 1] = tg / tw, out[p0 * 4 + 2] = tb / tw, out[p0 * 4 + 3] = T(0);
        }
}

}  // namespace

extern "C" {
int orc_blur_f32(const float* in, const float* depth, uint32_t W, uint32_t H, float* out) {
    std::vector<float> tmp(size_t(W) * H * 4);
    blur_pass_impl<float>(in, depth, W, H, 0, tmp.data());
    blur_pass_impl<float>(tmp.data(), depth, W, H, 1, out);
    return 0;
}
int orc_blur_f64(const double* in, const float* depth, uint32_t W, uint32_t H, double* out) {
    std::vector<double> tmp(size_t(W) * H * 4);
    blur_pass_impl<double>(in, depth, W, H, 0, tmp.data());
    blur_pass_impl<double>(tmp.data(), depth, W, H, 1, out);
    return 0;
}
float orc_exp2_poly(float t) { return exp2_poly32(t); }
}  // extern "C"
