// cull_shim.cpp -- C entry points into the C++ adapter's culling helpers (include/f184gi_foreground.hpp), so that
// a test can hold them against the reference's own tc::Frustum / tc::BoundingBox on the same inputs.
#include <cstring>
#include <vector>

#include "f184gi_foreground.hpp"

using namespace Foreground;

static f184gi_bounds box_of(const float mn[3], const float mx[3]) {
    return {{mn[0], mn[1], mn[2]}, 0.0f, {mx[0], mx[1], mx[2]}, 0.0f};
}

extern "C" {

int cull_define(const float proj[16], void* out) {
    GIFrustum f;
    int rc = GIFrustumDefine(proj, &f);
    std::memcpy(out, &f, sizeof f);
    return rc;
}

void cull_transformed(const void* in, const float m12[12], void* out) {
    GIFrustum f;
    GIMatrix3x4 m;
    std::memcpy(&f, in, sizeof f);
    std::memcpy(m.m, m12, 48);
    GIFrustum t = GIFrustumTransformed(f, m);
    std::memcpy(out, &t, sizeof t);
}

void cull_bounds_transformed(const float mn[3], const float mx[3], const float m12[12], float out[6]) {
    GIMatrix3x4 m;
    std::memcpy(m.m, m12, 48);
    f184gi_bounds r = GIBoundsTransformed(box_of(mn, mx), m);
    out[0] = r.min.x, out[1] = r.min.y, out[2] = r.min.z, out[3] = r.max.x, out[4] = r.max.y, out[5] = r.max.z;
}

int cull_inside_fast(const void* in, const float mn[3], const float mx[3]) {
    GIFrustum f;
    std::memcpy(&f, in, sizeof f);
    return int(GIIsInsideFast(f, box_of(mn, mx)));
}

// CullList over n primitives, each a single triangle list given by its object-space box (boxes: n x 6 floats,
// mats: n x 12); keep[i] = 1 when pair i survives.  Every other primitive carries no box, so its bounds come from
// its vertices: a two-triangle soup spanning the box's corners.
void cull_list(const void* frustum, uint32_t n, const float* mats, const float* boxes, uint8_t* keep) {
    GIFrustum f;
    std::memcpy(&f, frustum, sizeof f);
    std::vector<f184gi_bounds> b(n);
    std::vector<float> soup(size_t(n) * 18);
    std::vector<GIPrimitive> prims(n);
    std::vector<const GIPrimitive*> list(n);
    std::vector<GIMatrix3x4> ms(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* bx = boxes + size_t(i) * 6;
        b[i] = box_of(bx, bx + 3);
        float* s = soup.data() + size_t(i) * 18;
        const float tri[18] = {bx[0], bx[1], bx[2], bx[3], bx[1], bx[2], bx[3], bx[4], bx[2],
                               bx[0], bx[4], bx[5], bx[3], bx[4], bx[5], bx[0], bx[1], bx[5]};
        std::memcpy(s, tri, sizeof tri);
        prims[i] = {s, nullptr, 2, (i & 1) ? &b[i] : nullptr};
        list[i] = &prims[i];
        std::memcpy(ms[i].m, mats + size_t(i) * 12, 48);
    }
    std::vector<GIMatrix3x4> km;
    std::vector<const GIPrimitive*> kp;
    CullList(f, ms, list, km, kp);
    std::memset(keep, 0, n);
    for (const GIPrimitive* p : kp) keep[p - prims.data()] = 1;
}

}  // extern "C"
