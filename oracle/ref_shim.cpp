// ref_shim.cpp -- C entry points into the reference's own Math library and CCamera, compiled from the
// reference sources (see build.py).  TEST INFRASTRUCTURE ONLY: it pins the boundary types and the camera
// conventions that the product's host helpers restate.
#include <cstring>

#include "BoundingBox.h"
#include "Color.h"
#include "Camera.h"
#include "Frustum.h"
#include "Matrix3x4.h"
#include "Matrix4.h"
#include "Quaternion.h"
#include "Vector3.h"

extern "C" {

// 0 Vector3, 1 BoundingBox, 2 Frustum, 3 Matrix4, 4 Matrix3x4, 5 Color
int ref_sizeof(int which) {
    switch (which) {
        case 0: return int(sizeof(tc::Vector3));
        case 1: return int(sizeof(tc::BoundingBox));
        case 2: return int(sizeof(tc::Frustum));
        case 3: return int(sizeof(tc::Matrix4));
        case 4: return int(sizeof(tc::Matrix3x4));
        case 5: return int(sizeof(tc::Color));
        default: return -1;
    }
}

void ref_calc_perspective(float fovy, float aspect, float n, float f, float out[16]) {
    Foreground::CCamera cam(false);
    cam.SetFovY(fovy);
    cam.SetAspectRatio(aspect);
    cam.SetNearClip(n);
    cam.SetFarClip(f);
    std::memcpy(out, cam.GetMatrix().Data(), 64);
}

void ref_calc_ortho(float mx, float my, float n, float f, float out[16]) {
    Foreground::CCamera cam(true);
    cam.SetMagX(mx);
    cam.SetMagY(my);
    cam.SetNearClip(n);
    cam.SetFarClip(f);
    std::memcpy(out, cam.GetMatrix().Data(), 64);
}

void ref_matrix4_inverse(const float in[16], float out[16]) {
    tc::Matrix4 m(in);
    std::memcpy(out, m.Inverse().Data(), 64);
}

// BoundingBox(min, max).Transformed(Matrix3x4(m12)) -> out min[3], max[3]
void ref_bbox_transformed(const float mn[3], const float mx[3], const float m12[12], float out[6]) {
    tc::BoundingBox b(tc::Vector3(mn[0], mn[1], mn[2]), tc::Vector3(mx[0], mx[1], mx[2]));
    tc::Matrix3x4 m(m12);
    tc::BoundingBox r = b.Transformed(m);
    out[0] = r.Min.x, out[1] = r.Min.y, out[2] = r.Min.z;
    out[3] = r.Max.x, out[4] = r.Max.y, out[5] = r.Max.z;
}

// Frustum::Define(projection) then IsInsideFast(box) in view space: 0 outside, 1 intersects, 2 inside
int ref_frustum_box(const float proj[16], const float mn[3], const float mx[3]) {
    tc::Frustum fr;
    fr.Define(tc::Matrix4(proj));
    tc::BoundingBox b(tc::Vector3(mn[0], mn[1], mn[2]), tc::Vector3(mx[0], mx[1], mx[2]));
    return int(fr.IsInsideFast(b));
}

static_assert(sizeof(tc::Frustum) == 264, "tc::Frustum: 6 planes of 28 bytes, 8 corners of 12");

// Frustum::Define(projection), its 264 bytes (planes, then corners)
void ref_frustum_define(const float proj[16], void* out) {
    tc::Frustum fr;
    fr.Define(tc::Matrix4(proj));
    std::memcpy(out, &fr, sizeof fr);
}

// a Frustum given as its 264 bytes, Transformed(Matrix3x4(m12)) -> 264 bytes
void ref_frustum_transformed(const void* in, const float m12[12], void* out) {
    tc::Frustum fr;
    std::memcpy(static_cast<void*>(&fr), in, sizeof fr);
    tc::Frustum t = fr.Transformed(tc::Matrix3x4(m12));
    std::memcpy(out, &t, sizeof t);
}

// a Frustum given as its 264 bytes, IsInsideFast(BoundingBox(mn, mx)): 0 outside, 2 inside
int ref_frustum_inside_fast(const void* in, const float mn[3], const float mx[3]) {
    tc::Frustum fr;
    std::memcpy(static_cast<void*>(&fr), in, sizeof fr);
    return int(fr.IsInsideFast(tc::BoundingBox(tc::Vector3(mn[0], mn[1], mn[2]), tc::Vector3(mx[0], mx[1], mx[2]))));
}

// q(ex, ey, ez) * v for the Euler-angle constructor (degrees) of tc::Quaternion
void ref_quat_euler_rotate(float ex, float ey, float ez, const float v[3], float out[3]) {
    tc::Vector3 r = tc::Quaternion(ex, ey, ez) * tc::Vector3(v[0], v[1], v[2]);
    out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

// tc::Matrix3x4(translation, rotation (w, x, y, z), scale), row-major 3x4
void ref_matrix_trs(const float t[3], const float q[4], const float s[3], float out[12]) {
    tc::Matrix3x4 m(tc::Vector3(t[0], t[1], t[2]), tc::Quaternion(q[0], q[1], q[2], q[3]), tc::Vector3(s[0], s[1], s[2]));
    std::memcpy(out, m.Data(), 12 * sizeof(float));
}

}  // extern "C"
