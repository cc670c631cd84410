// scene.cpp -- seeded synthetic scenes and the camera helpers of the reference's CCamera.
//
// Scenes stand in for the reference's glTF import (Foreground/SceneGraph/glTFSceneImporter.cpp:200-330): a room
// of six quads bounding [-10,10]^3 (the ceiling covers half the room, leaving an opening for the sun) plus
// boxes and UV-spheres, per-triangle RGBA8 albedo and roughness, one directional light with the reference sun's colour (App/MainBehaviour.cpp:40-42) and a camera inside the room.
// Random numbers: splitmix64 seeding xoshiro256**; object j draws from its own sub-stream.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gi_internal.h"

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform in [0, 1), 24 random bits: exact in FP32
    float uni() { return float(next() >> 40) * (1.0f / 16777216.0f); }
    float uni(float a, float b) { return a + (b - a) * uni(); }
};

uint64_t substream(uint64_t seed, uint64_t j) {
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (j + 1));
    return Rng::splitmix(x);
}

struct Builder {
    std::vector<float> xyz;
    std::vector<uint32_t> albedo;
    std::vector<float> rough;
    void tri(const float* a, const float* b, const float* c, Rng& r) {
        xyz.insert(xyz.end(), {a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2]});
        uint32_t rgb = uint32_t(r.next() >> 40) & 0xffffffu;
        albedo.push_back(rgb | 0xff000000u);
        rough.push_back(r.uni(0.1f, 0.9f));
    }
};

void rotate(const float q[4], const float v[3], float out[3]) {
    // q = (x, y, z, w) unit quaternion; out = q v q*
    float x = q[0], y = q[1], z = q[2], w = q[3];
    float tx = 2.0f * (y * v[2] - z * v[1]);
    float ty = 2.0f * (z * v[0] - x * v[2]);
    float tz = 2.0f * (x * v[1] - y * v[0]);
    out[0] = v[0] + w * tx + (y * tz - z * ty);
    out[1] = v[1] + w * ty + (z * tx - x * tz);
    out[2] = v[2] + w * tz + (x * ty - y * tx);
}

void add_room(Builder& b, Rng& r) {
    const float L = 10.0f;
    // six quads (two triangles each): walls and floor bound [-L, L]^3; the ceiling spans x in [-L, 0] only,
    // and the opening over x in [0, L] lets the sun into the room
    const float q[6][4][3] = {
        {{-L, -L, -L}, {-L, L, -L}, {-L, L, L}, {-L, -L, L}},  // -x wall
        {{L, -L, -L}, {L, -L, L}, {L, L, L}, {L, L, -L}},      // +x wall
        {{-L, -L, -L}, {-L, -L, L}, {L, -L, L}, {L, -L, -L}},  // floor
        {{-L, L, -L}, {0, L, -L}, {0, L, L}, {-L, L, L}},      // ceiling (half)
        {{-L, -L, -L}, {L, -L, -L}, {L, L, -L}, {-L, L, -L}},  // -z wall
        {{-L, -L, L}, {-L, L, L}, {L, L, L}, {L, -L, L}},      // +z wall
    };
    for (const auto& f : q) {
        b.tri(f[0], f[1], f[2], r);
        b.tri(f[0], f[2], f[3], r);
    }
}

void add_box(Builder& b, Rng& r, const float ctr[3], float half, const float q[4]) {
    float c[8][3];
    for (int i = 0; i < 8; ++i) {
        float v[3] = {(i & 1) ? half : -half, (i & 2) ? half : -half, (i & 4) ? half : -half};
        float o[3];
        rotate(q, v, o);
        for (int a = 0; a < 3; ++a) c[i][a] = ctr[a] + o[a];
    }
    const int f[6][4] = {{0, 2, 6, 4}, {1, 5, 7, 3}, {0, 4, 5, 1}, {2, 3, 7, 6}, {0, 1, 3, 2}, {4, 6, 7, 5}};
    for (auto& qd : f) {
        b.tri(c[qd[0]], c[qd[1]], c[qd[2]], r);
        b.tri(c[qd[0]], c[qd[2]], c[qd[3]], r);
    }
}

void add_sphere(Builder& b, Rng& r, const float ctr[3], float rad, int stacks, int slices) {
    auto vert = [&](int i, int j, float* o) {
        double th = M_PI * double(i) / double(stacks);
        double ph = 2.0 * M_PI * double(j % slices) / double(slices);
        o[0] = ctr[0] + float(rad * std::sin(th) * std::cos(ph));
        o[1] = ctr[1] + float(rad * std::cos(th));
        o[2] = ctr[2] + float(rad * std::sin(th) * std::sin(ph));
    };
    for (int i = 0; i < stacks; ++i)
        for (int j = 0; j < slices; ++j) {
            float a[3], bb[3], c[3], d[3];
            vert(i, j, a);
            vert(i + 1, j, bb);
            vert(i + 1, j + 1, c);
            vert(i, j + 1, d);
            if (i != 0) b.tri(a, bb, d, r);
            if (i != stacks - 1) b.tri(d, bb, c, r);
        }
}

}  // namespace

extern "C" {

int f184gi_scene_generate(uint64_t seed, uint64_t target_tris, uint32_t nobjects, f184gi_scene** out) {
    if (!out) return f184::fail(F184GI_ERR_INVALID, "scene_generate: out is null");
    *out = nullptr;
    if (target_tris < 12 || target_tris > (uint64_t(1) << 31))
        return f184::fail(F184GI_ERR_INVALID, "scene_generate: target_tris out of range");
    Builder b;
    b.xyz.reserve(target_tris * 9 + 1024);
    std::vector<uint32_t> first, count;
    {
        Rng r(substream(seed, 0));
        first.push_back(0);
        add_room(b, r);
        count.push_back(12);
    }
    uint32_t nbox = (nobjects + 1) / 2, nsph = nobjects / 2;
    double budget = nsph ? (double(target_tris) - 12.0 - 12.0 * nbox) / double(nsph) : 0.0;
    int stacks = std::max(3, int(std::lround(std::sqrt(std::max(budget, 0.0) / 4.0))));
    int slices = std::max(3, int(std::lround(std::max(budget, 0.0) / (2.0 * (stacks - 1)))));
    // object sizes shrink with the count so that every scene fills about the same share of the room as the
    // 200-object one (~16% of its volume), whatever the number of objects
    const float size_scale = nobjects > 200 ? float(std::cbrt(200.0 / double(nobjects))) : 1.0f;
    for (uint32_t j = 0; j < nobjects; ++j) {
        Rng r(substream(seed, j + 1));
        bool box = (j % 2) == 0;
        float half = r.uni(0.3f, 1.5f) * size_scale;
        float reach = box ? half * 1.7320508f : half;
        float ctr[3];
        for (int a = 0; a < 3; ++a) ctr[a] = r.uni(-10.0f + reach + 0.05f, 10.0f - reach - 0.05f);
        first.push_back(uint32_t(b.albedo.size()));
        if (box) {
            float q[4];
            float n = 0.0f;
            for (int a = 0; a < 4; ++a) {
                q[a] = r.uni(-1.0f, 1.0f);
                n += q[a] * q[a];
            }
            n = std::sqrt(std::max(n, 1e-12f));
            for (int a = 0; a < 4; ++a) q[a] /= n;
            add_box(b, r, ctr, half, q);
        } else {
            add_sphere(b, r, ctr, half, stacks, slices);
        }
        count.push_back(uint32_t(b.albedo.size()) - first.back());
    }
    f184gi_scene* s = static_cast<f184gi_scene*>(std::calloc(1, sizeof(f184gi_scene)));
    if (!s) return f184::fail(F184GI_ERR_OOM, "scene_generate: host allocation failed");
    s->ntris = b.albedo.size();
    s->nobjects = uint32_t(first.size());
    s->tri_xyz = static_cast<float*>(std::malloc(b.xyz.size() * 4));
    s->albedo = static_cast<uint32_t*>(std::malloc(b.albedo.size() * 4));
    s->roughness = static_cast<float*>(std::malloc(b.rough.size() * 4));
    s->object_first = static_cast<uint32_t*>(std::malloc(first.size() * 4));
    s->object_count = static_cast<uint32_t*>(std::malloc(count.size() * 4));
    if (!s->tri_xyz || !s->albedo || !s->roughness || !s->object_first || !s->object_count) {
        f184gi_scene_free(s);
        return f184::fail(F184GI_ERR_OOM, "scene_generate: host allocation failed");
    }
    std::memcpy(s->tri_xyz, b.xyz.data(), b.xyz.size() * 4);
    std::memcpy(s->albedo, b.albedo.data(), b.albedo.size() * 4);
    std::memcpy(s->roughness, b.rough.data(), b.rough.size() * 4);
    std::memcpy(s->object_first, first.data(), first.size() * 4);
    std::memcpy(s->object_count, count.data(), count.size() * 4);
    s->bounds.min = {-10.0f, -10.0f, -10.0f};
    s->bounds.max = {10.0f, 10.0f, 10.0f};
    {
        Rng r(substream(seed, 0xFFFFFFFFull));
        // sun colour and intensity of the reference's directional light (MainBehaviour.cpp:40-42)
        s->light.luminance[0] = 1.1f * 4.0f;
        s->light.luminance[1] = 0.93f * 4.0f;
        s->light.luminance[2] = 0.81f * 4.0f;
        float cy = r.uni(0.3f, 1.0f), ph = r.uni(0.0f, 6.2831853f);
        float sy = std::sqrt(1.0f - cy * cy);
        // direction of travel: from the upper hemisphere downwards
        s->light.direction[0] = -sy * std::cos(ph);
        s->light.direction[1] = -cy;
        s->light.direction[2] = -sy * std::sin(ph);
    }
    f184gi_scene_camera(s, seed, 0, s->eye, s->target);
    *out = s;
    return F184GI_OK;
}

void f184gi_scene_free(f184gi_scene* s) {
    if (!s) return;
    std::free(s->tri_xyz);
    std::free(s->albedo);
    std::free(s->roughness);
    std::free(s->object_first);
    std::free(s->object_count);
    std::free(s);
}

int f184gi_scene_camera(const f184gi_scene* s, uint64_t seed, uint32_t i, float eye[3], float target[3]) {
    if (!s || !eye || !target) return f184::fail(F184GI_ERR_INVALID, "scene_camera: null argument");
    Rng r(substream(seed ^ 0x5EED5EEDull, 0x10000000ull + i));
    // the eye sits in free space: at least 0.5 m outside every object's bounding box (up to 256 draws)
    std::vector<float> box(size_t(s->nobjects) * 6);
    for (uint32_t o = 0; o < s->nobjects; ++o) {
        float* bb = &box[size_t(o) * 6];
        for (int a = 0; a < 3; ++a) bb[a] = 1e30f, bb[3 + a] = -1e30f;
        if (o == 0) continue;  // the room itself
        const float* p = s->tri_xyz + uint64_t(s->object_first[o]) * 9;
        for (uint64_t v = 0; v < uint64_t(s->object_count[o]) * 3; ++v)
            for (int a = 0; a < 3; ++a) {
                bb[a] = std::min(bb[a], p[v * 3 + a]);
                bb[3 + a] = std::max(bb[3 + a], p[v * 3 + a]);
            }
    }
    for (int attempt = 0; attempt < 256; ++attempt) {
        eye[0] = r.uni(-8.0f, 8.0f);
        eye[1] = r.uni(-6.0f, 6.0f);
        eye[2] = r.uni(-8.0f, 8.0f);
        bool clear = true;
        for (uint32_t o = 1; o < s->nobjects && clear; ++o) {
            const float* bb = &box[size_t(o) * 6];
            bool inside = true;
            for (int a = 0; a < 3; ++a) inside = inside && eye[a] > bb[a] - 0.5f && eye[a] < bb[3 + a] + 0.5f;
            clear = !inside;
        }
        if (clear) break;
    }
    float d[3];
    float n;
    do {
        for (int a = 0; a < 3; ++a) d[a] = r.uni(-1.0f, 1.0f);
        n = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    } while (n < 0.05f || n > 1.0f);
    n = std::sqrt(n);
    d[1] *= 0.5f;  // keep views closer to horizontal
    for (int a = 0; a < 3; ++a) target[a] = eye[a] + 5.0f * d[a] / n;
    return F184GI_OK;
}

int f184gi_scene_move_objects(f184gi_scene* s, uint64_t seed, float fraction, float max_offset,
                              uint32_t* moved_out, uint32_t* nmoved) {
    if (!s || !nmoved) return f184::fail(F184GI_ERR_INVALID, "scene_move_objects: null argument");
    *nmoved = 0;
    if (s->nobjects <= 1 || fraction <= 0.0f) return F184GI_OK;
    Rng r(substream(seed ^ 0x0B1EC7ull, 0x20000000ull));
    uint32_t nobj = s->nobjects - 1;  // object 0 is the room
    uint32_t k = std::min<uint32_t>(nobj, std::max<uint32_t>(1u, uint32_t(std::lround(double(fraction) * nobj))));
    std::vector<uint32_t> ids(nobj);
    for (uint32_t i = 0; i < nobj; ++i) ids[i] = i + 1;
    for (uint32_t i = 0; i < k; ++i) {  // partial Fisher-Yates
        uint32_t j = i + uint32_t(r.next() % (nobj - i));
        std::swap(ids[i], ids[j]);
    }
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t o = ids[i];
        float* p = s->tri_xyz + uint64_t(s->object_first[o]) * 9;
        uint64_t nv = uint64_t(s->object_count[o]) * 3;
        float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
        for (uint64_t v = 0; v < nv; ++v)
            for (int a = 0; a < 3; ++a) {
                mn[a] = std::min(mn[a], p[v * 3 + a]);
                mx[a] = std::max(mx[a], p[v * 3 + a]);
            }
        float off[3];
        for (int a = 0; a < 3; ++a) {
            off[a] = r.uni(-max_offset, max_offset);
            // stay inside the room
            off[a] = std::min(off[a], 9.95f - mx[a]);
            off[a] = std::max(off[a], -9.95f - mn[a]);
        }
        for (uint64_t v = 0; v < nv; ++v)
            for (int a = 0; a < 3; ++a) p[v * 3 + a] += off[a];
        if (moved_out) moved_out[i] = o;
    }
    *nmoved = k;
    return F184GI_OK;
}

// CCamera::CalcPerspective, Foreground/SceneGraph/Camera.cpp:85-102 (same FP32 arithmetic; Vulkan y flip)
void f184gi_camera_perspective(float fovy, float aspect, float n, float f, float out[16]) {
    const float kPi = 3.14159265358979323846f;
    float rad = fovy / 180.f * kPi;
    float ys = float(std::tan(double(rad / 2)));
    float xs = ys * aspect;
    float right = xs * n, top = ys * n;
    float a = n / right, b = n / top;
    float c = (f + n) / (n - f);
    float d = -2 * f * n / (f - n);
    const float m[16] = {a, 0, 0, 0, 0, -b, 0, 0, 0, 0, c, d, 0, 0, -1, 0};
    std::memcpy(out, m, sizeof(m));
}

// CCamera::CalcOrtho, Camera.cpp:104-111
void f184gi_camera_ortho(float mx, float my, float n, float f, float out[16]) {
    float a = 1.0f / mx, b = 1.0f / my, c = 1.0f / (n - f), d = n / (n - f);
    const float m[16] = {a, 0, 0, 0, 0, b, 0, 0, 0, 0, c, d, 0, 0, 0, 1};
    std::memcpy(out, m, sizeof(m));
}

void f184gi_camera_look_at(const float eye[3], const float target[3], float out[16]) {
    double f[3] = {double(target[0]) - eye[0], double(target[1]) - eye[1], double(target[2]) - eye[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& v : f) v /= fl;
    double up[3] = {0.0, 1.0, 0.0};
    if (std::fabs(f[1]) > 0.999) up[1] = 0.0, up[2] = 1.0;
    // right = f x up, true up = right x f; camera basis: x = right, y = up, z = -f
    double rgt[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    double rl = std::sqrt(rgt[0] * rgt[0] + rgt[1] * rgt[1] + rgt[2] * rgt[2]);
    for (double& v : rgt) v /= rl;
    double u[3] = {rgt[1] * f[2] - rgt[2] * f[1], rgt[2] * f[0] - rgt[0] * f[2], rgt[0] * f[1] - rgt[1] * f[0]};
    double z[3] = {-f[0], -f[1], -f[2]};
    const double* rows[3] = {rgt, u, z};
    for (int r = 0; r < 3; ++r) {
        out[r * 4 + 0] = float(rows[r][0]);
        out[r * 4 + 1] = float(rows[r][1]);
        out[r * 4 + 2] = float(rows[r][2]);
        out[r * 4 + 3] = float(-(rows[r][0] * eye[0] + rows[r][1] * eye[1] + rows[r][2] * eye[2]));
    }
    out[12] = out[13] = out[14] = 0.0f;
    out[15] = 1.0f;
}

int f184gi_mat4_inverse(const float m[16], float out[16]) {
    double a[16], inv[16];
    for (int i = 0; i < 16; ++i) a[i] = m[i];
    if (!f184::invert4(a, inv)) return f184::fail(F184GI_ERR_INVALID, "mat4_inverse: singular matrix");
    for (int i = 0; i < 16; ++i) out[i] = float(inv[i]);
    return F184GI_OK;
}

}  // extern "C"
