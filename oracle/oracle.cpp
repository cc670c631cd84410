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

// Snapped triangle: vertices in 1/16 pixel, depth plane z(X, Y) = z0 + a (X - X0) + b (Y - Y0) with
// z0, a, b rounded to FP32 from an FP64 plane solve.
struct SnapTri {
    int64_t X[3], Y[3];
    double Z[3];
    int64_t area2;
    float z0, a, b;
    int64_t x0, x1, y0, y1;  // pixel range, inclusive
};

bool snap_tri(const V4& a, const V4& b, const V4& c, uint32_t W, uint32_t H, SnapTri& s) {
    const V4* v[3] = {&a, &b, &c};
    for (int i = 0; i < 3; ++i) {
        if (!(v[i]->w > 0.0)) return false;
        double nx = v[i]->x / v[i]->w, ny = v[i]->y / v[i]->w, nz = v[i]->z / v[i]->w;
        s.X[i] = std::llrint((nx + 1.0) * (8.0 * double(W)));
        s.Y[i] = std::llrint((ny + 1.0) * (8.0 * double(H)));
        s.Z[i] = nz;
    }
    int64_t area2 = (s.X[1] - s.X[0]) * (s.Y[2] - s.Y[0]) - (s.Y[1] - s.Y[0]) * (s.X[2] - s.X[0]);
    if (area2 == 0) return false;
    if (area2 < 0) {
        std::swap(s.X[1], s.X[2]);
        std::swap(s.Y[1], s.Y[2]);
        std::swap(s.Z[1], s.Z[2]);
        area2 = -area2;
    }
    s.area2 = area2;
    {
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

template <class T>
void cone(const Chain<T>& ch, Vec3<T> o, Vec3<T> dir, T tan_half, const f184gi_cone_params& p, T tmax,
          T out[4]) {
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

template <class T>
int trace_impl(const f184gi_grid_frame* frame, uint32_t dim, uint32_t levels, uint32_t aniso, const T* chain,
               const float view[16], const float proj[16], uint32_t W, uint32_t H, const float* depth,
               const uint32_t* normal, const uint16_t* rough, const f184gi_cone_params* params, T* out,
               uint32_t row_begin, uint32_t row_end, int nthreads) {
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
                if (std::is_same<T, float>::value) {
                    // the device arithmetic: the projective rows (z, w) in FP64, x and y in FP32
                    const double dnx = double(nx), dny = double(ny), ddz = double(nz);
                    const double vz = IP[8] * dnx + IP[9] * dny + IP[10] * ddz + IP[11];
                    const double vw = IP[12] * dnx + IP[13] * dny + IP[14] * ddz + IP[15];
                    const double rw = 1.0 / vw;
                    cs = Vec3<T>{vp[0] * T(rw), vp[1] * T(rw), T(vz * rw)};
                }
                Vec3<T> wp{iv[0] * cs.x + iv[1] * cs.y + iv[2] * cs.z + iv[3],
                           iv[4] * cs.x + iv[5] * cs.y + iv[6] * cs.z + iv[7],
                           iv[8] * cs.x + iv[9] * cs.y + iv[10] * cs.z + iv[11]};
                Vec3<T> nv = oct_decode<T>(normal[pi]);
                Vec3<T> nw = vnorm(Vec3<T>{iv[0] * nv.x + iv[1] * nv.y + iv[2] * nv.z,
                                           iv[4] * nv.x + iv[5] * nv.y + iv[6] * nv.z,
                                           iv[8] * nv.x + iv[9] * nv.y + iv[10] * nv.z});
                T r = T(h2f(rough[pi]));
                Vec3<T> pv = vmul(vsub(wp, org), inv_vs);
                Vec3<T> o = vadd(pv, vmul(nw, T(p.start_offset)));
                Vec3<T> bx, by, bz;
                make_coord_space(nw, bx, by, bz);
                T acc[4] = {T(0), T(0), T(0), T(0)};
                if (p.diffuse_cones >= 5) {
                    T c0[4];
                    cone(ch, o, bz, T(p.diffuse_tan_half), p, tmax, c0);
                    for (int k = 0; k < 4; ++k) acc[k] += T(0.25) * c0[k];
                    const T cphi[4] = {T(1), T(0), T(-1), T(0)}, sphi[4] = {T(0), T(1), T(0), T(-1)};
                    for (int s = 0; s < 4; ++s) {
                        Vec3<T> side = vadd(vmul(bx, cphi[s]), vmul(by, sphi[s]));
                        Vec3<T> d = vnorm(vadd(vmul(bz, ct), vmul(side, st)));
                        T cs4[4];
                        cone(ch, o, d, T(p.diffuse_tan_half), p, tmax, cs4);
                        for (int k = 0; k < 4; ++k) acc[k] += T(0.1875) * cs4[k];
                    }
                } else {
                    cone(ch, o, bz, T(p.diffuse_tan_half), p, tmax, acc);
                }
                for (int k = 0; k < 4; ++k) od[k] = acc[k];
                if (p.specular) {
                    Vec3<T> vdir = vnorm(vsub(wp, eye));
                    T dn = vdot(vdir, nw);
                    Vec3<T> rd = vnorm(vsub(vdir, vmul(nw, T(2) * dn)));
                    T th = std::max(r, T(p.min_spec_tan_half));
                    T sc[4];
                    cone(ch, o, rd, th, p, tmax, sc);
                    for (int k = 0; k < 4; ++k) os[k] = sc[k];
                }
            }
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
    for (uint64_t t = 0; t < ntris; ++t) {
        const float* p = tri + t * 9;
        V4 poly[12];
        bool inside = true;
        for (int v = 0; v < 3; ++v) {
            double x = p[v * 3], y = p[v * 3 + 1], z = p[v * 3 + 2];
            poly[v] = {mrow(M, x, y, z), mrow(M + 4, x, y, z), mrow(M + 8, x, y, z), mrow(M + 12, x, y, z)};
            for (int k = 0; k < 6; ++k)
                if (!(plane_dist(k, poly[v]) >= 0.0)) inside = false;
        }
        int n = 3;
        if (!inside) n = clip_polygon(poly, 3);
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
