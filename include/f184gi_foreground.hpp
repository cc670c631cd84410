// f184gi_foreground.hpp -- C++ host adapter with the reference renderer's pass shape (header-only).
//
// Mirrors how CMegaPipeline::Render drives the GI passes (Foreground/Renderer/MegaPipeline.cpp:188-268):
//   RenderList(modelMats, primitives)  <- CZOnlyRenderer::RenderList + CVoxelizeRenderer::RenderList
//                                          (ZOnlyRenderer.h:21-22, VoxelizeRenderer.h:21-22): one (Matrix3x4,
//                                          primitive) pair per visible primitive, as CSceneView hands them out
//                                          (SceneView.h:29-33)
//   BuildMips()                         <- no reference counterpart (its volume has one level)
//   TraceViews(views)                   <- the lighting_indirect pass (MegaPipeline.cpp:241-268)
//   CullList(frustum, ...)              <- CSceneView::PrepareToRender's frustum branch (SceneView.cpp:32-40):
//                                          the camera frustum in world space, each object's world bounds tested
//                                          with Frustum::IsInsideFast (Octree.cpp:105-116)
// Primitive geometry is uploaded once and kept on the device, keyed by the primitive's address (the reference
// caches per-primitive pipeline resources the same way, VoxelizeRenderer.h:47-49).  Errors come back as the C ABI's
// status codes (the reference returns silently; this adapter does not).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>

#include "f184gi.h"

namespace Foreground {

// Layout of tc::Matrix3x4 (Math/Matrix3x4.h): 12 floats, row-major, acting on column vectors.
struct GIMatrix3x4 {
    float m[12];
};
static_assert(sizeof(GIMatrix3x4) == 48, "tc::Matrix3x4 is 48 bytes");
// Layout of tc::Matrix4 (Math/Matrix4.h): 16 floats, row-major; f184gi_view's view/proj and GIFrustumDefine take it.
struct GIMatrix4 {
    float m[16];
};
static_assert(sizeof(GIMatrix4) == 64, "tc::Matrix4 is 64 bytes");
static_assert(sizeof(f184gi_vec3) == 12, "tc::Vector3 is 12 bytes");
static_assert(sizeof(f184gi_bounds) == 32, "tc::BoundingBox is 32 bytes");

// Object-space triangle soup of one primitive (host memory, 9 floats per triangle) with per-triangle RGBA8 albedo.
// `bounds` is its object-space box for culling; when null, CullList takes the box of the vertices.
struct GIPrimitive {
    const float* xyz;
    const uint32_t* albedo;
    uint64_t ntris;
    const f184gi_bounds* bounds = nullptr;
};

// ---- view culling: the reference's Math types and the steps of its tests, restated ----
// The arithmetic follows the reference's scalar (non-SSE) code operation by operation, so that compiled without
// floating-point contraction the planes, boxes and decisions are bit-identical to tc::Frustum / tc::BoundingBox.

// Layout of tc::Plane (Math/Plane.h:116-122): unit normal, its component-wise absolute value, and d; points p
// with normal . p + d >= 0 are on the inner side.
struct GIPlane {
    f184gi_vec3 normal;
    f184gi_vec3 absNormal;
    float d;
};
// Layout of tc::Frustum (Math/Frustum.h:35-43, 180-182): the near, left, right, up, down and far planes, then
// eight corners, 0..3 on the near face and 4..7 on the far face, (+x +y), (+x -y), (-x -y), (-x +y) in each.
struct GIFrustum {
    GIPlane planes[6];
    f184gi_vec3 vertices[8];
};
static_assert(sizeof(GIPlane) == 28, "tc::Plane is 28 bytes");
static_assert(sizeof(GIFrustum) == 264, "tc::Frustum is 264 bytes");

// tc::Intersection (Math/MathDefs.h:64-69); IsInsideFast answers OUTSIDE or INSIDE only.
enum GIIntersection { GI_OUTSIDE = 0, GI_INTERSECTS = 1, GI_INSIDE = 2 };

namespace gi_detail {
inline f184gi_vec3 affine(const float* m, f184gi_vec3 v) {  // Matrix3x4 * Vector3 (Math/Matrix3x4.h:275-279)
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3], m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7],
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11]};
}
inline f184gi_vec3 project(const float* m, f184gi_vec3 v) {  // Matrix4 * Vector3, divided by w (Matrix4.h:279-285)
    float inv_w = 1.0f / (m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15]);
    return {(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3]) * inv_w, (m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7]) * inv_w,
            (m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11]) * inv_w};
}
inline float dot(f184gi_vec3 a, f184gi_vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// Plane::Define(v0, v1, v2) (Math/Plane.h:65-79): normal = (v1 - v0) x (v2 - v0), normalized unless its squared
// length is zero or within float epsilon of one (Vector3::Normalized, Vector3.h:432-442), through v0.
inline GIPlane plane(f184gi_vec3 a, f184gi_vec3 b, f184gi_vec3 c) {
    f184gi_vec3 u{b.x - a.x, b.y - a.y, b.z - a.z}, w{c.x - a.x, c.y - a.y, c.z - a.z};
    f184gi_vec3 n{u.y * w.z - u.z * w.y, u.z * w.x - u.x * w.z, u.x * w.y - u.y * w.x};
    const float len2 = dot(n, n), eps = std::numeric_limits<float>::epsilon();
    if (!(len2 + eps >= 1.0f && len2 - eps <= 1.0f) && len2 > 0.0f) {
        const float s = 1.0f / std::sqrt(len2);
        n = {n.x * s, n.y * s, n.z * s};
    }
    return {n, {std::fabs(n.x), std::fabs(n.y), std::fabs(n.z)}, -dot(n, a)};
}
}  // namespace gi_detail

// Frustum::UpdatePlanes (Math/Frustum.cpp:225-244): the six planes from the corners; a mirroring transform leaves
// them facing out, which shows as far corner 5 behind the near plane, and then all six are flipped.
inline void GIUpdatePlanes(GIFrustum& f) {
    using gi_detail::plane;
    const f184gi_vec3* v = f.vertices;
    f.planes[0] = plane(v[2], v[1], v[0]);
    f.planes[1] = plane(v[3], v[7], v[6]);
    f.planes[2] = plane(v[1], v[5], v[4]);
    f.planes[3] = plane(v[0], v[4], v[7]);
    f.planes[4] = plane(v[6], v[5], v[1]);
    f.planes[5] = plane(v[5], v[6], v[7]);
    if (gi_detail::dot(f.planes[0].normal, v[5]) + f.planes[0].d < 0.0f)
        for (GIPlane& p : f.planes) {
            p.normal = {-p.normal.x, -p.normal.y, -p.normal.z};
            p.d = -p.d;
        }
}

// Frustum::Define(projection) (Math/Frustum.cpp:120-134): the NDC cube's corners (x, y in -1..1, depth 0..1)
// through the inverse of a row-major projection.  The inverse is f184gi_mat4_inverse (FP64 inside), so the
// corners agree with the reference's FP32 Matrix4::Inverse to rounding, not bit for bit.
inline int GIFrustumDefine(const float proj[16], GIFrustum* out) {
    float inv[16];
    int rc = f184gi_mat4_inverse(proj, inv);
    if (rc) return rc;
    const float xy[4][2] = {{1.0f, 1.0f}, {1.0f, -1.0f}, {-1.0f, -1.0f}, {-1.0f, 1.0f}};
    for (int i = 0; i < 8; ++i) out->vertices[i] = gi_detail::project(inv, {xy[i & 3][0], xy[i & 3][1], i < 4 ? 0.0f : 1.0f});
    GIUpdatePlanes(*out);
    return F184GI_OK;
}

// Frustum::Transformed(Matrix3x4) (Math/Frustum.cpp:199-207): corners through the transform, planes rebuilt --
// the camera-space frustum placed by the camera node's world transform.
inline GIFrustum GIFrustumTransformed(const GIFrustum& f, const GIMatrix3x4& m) {
    GIFrustum t;
    for (int i = 0; i < 8; ++i) t.vertices[i] = gi_detail::affine(m.m, f.vertices[i]);
    GIUpdatePlanes(t);
    return t;
}

// BoundingBox::Transformed(Matrix3x4) (Math/BoundingBox.cpp:157-166): the centre through the transform, the
// half-size through |rotation-scale|.
inline f184gi_bounds GIBoundsTransformed(const f184gi_bounds& b, const GIMatrix3x4& m) {
    const float* r = m.m;
    f184gi_vec3 c{(b.max.x + b.min.x) * 0.5f, (b.max.y + b.min.y) * 0.5f, (b.max.z + b.min.z) * 0.5f};
    f184gi_vec3 e{(b.max.x - b.min.x) * 0.5f, (b.max.y - b.min.y) * 0.5f, (b.max.z - b.min.z) * 0.5f};
    c = gi_detail::affine(r, c);
    f184gi_vec3 h{std::fabs(r[0]) * e.x + std::fabs(r[1]) * e.y + std::fabs(r[2]) * e.z,
                  std::fabs(r[4]) * e.x + std::fabs(r[5]) * e.y + std::fabs(r[6]) * e.z,
                  std::fabs(r[8]) * e.x + std::fabs(r[9]) * e.y + std::fabs(r[10]) * e.z};
    return {{c.x - h.x, c.y - h.y, c.z - h.z}, 0.0f, {c.x + h.x, c.y + h.y, c.z + h.z}, 0.0f};
}

// Frustum::IsInsideFast(BoundingBox) (Math/Frustum.h:142-157): OUTSIDE when the box lies wholly behind one plane,
// else INSIDE (boxes across a plane count as inside; the test never answers INTERSECTS).
inline GIIntersection GIIsInsideFast(const GIFrustum& f, const f184gi_bounds& b) {
    f184gi_vec3 c{(b.max.x + b.min.x) * 0.5f, (b.max.y + b.min.y) * 0.5f, (b.max.z + b.min.z) * 0.5f};
    f184gi_vec3 e{c.x - b.min.x, c.y - b.min.y, c.z - b.min.z};
    for (const GIPlane& p : f.planes) {
        float dist = gi_detail::dot(p.normal, c) + p.d;
        float reach = gi_detail::dot(p.absNormal, e);
        if (dist < -reach) return GI_OUTSIDE;
    }
    return GI_INSIDE;
}

// Object-space box of a primitive: its own `bounds`, else the box of its vertices.
inline f184gi_bounds GIPrimitiveBounds(const GIPrimitive& p) {
    if (p.bounds) return *p.bounds;
    const float inf = std::numeric_limits<float>::infinity();
    f184gi_bounds b{{inf, inf, inf}, 0.0f, {-inf, -inf, -inf}, 0.0f};
    for (uint64_t i = 0; i < p.ntris * 3; ++i) {
        const float* v = p.xyz + i * 3;
        b.min = {std::fmin(b.min.x, v[0]), std::fmin(b.min.y, v[1]), std::fmin(b.min.z, v[2])};
        b.max = {std::fmax(b.max.x, v[0]), std::fmax(b.max.y, v[1]), std::fmax(b.max.z, v[2])};
    }
    return b;
}

// The (model matrix, primitive) pairs whose world-space box is not wholly outside `frustum` (a world-space
// frustum, e.g. GIFrustumTransformed(camera frustum, camera world transform)), in their input order.
inline void CullList(const GIFrustum& frustum, const std::vector<GIMatrix3x4>& modelMats,
                     const std::vector<const GIPrimitive*>& primitives, std::vector<GIMatrix3x4>& keptMats,
                     std::vector<const GIPrimitive*>& keptPrims) {
    keptMats.clear();
    keptPrims.clear();
    for (size_t i = 0; i < primitives.size() && i < modelMats.size(); ++i) {
        const GIPrimitive* p = primitives[i];
        if (!p || p->ntris == 0) continue;
        if (GIIsInsideFast(frustum, GIBoundsTransformed(GIPrimitiveBounds(*p), modelMats[i])) == GI_OUTSIDE) continue;
        keptMats.push_back(modelMats[i]);
        keptPrims.push_back(p);
    }
}

class CVoxelGI {
public:
    CVoxelGI(const f184gi_grid_desc& desc, int device = 0, uint64_t hbm_budget = 0) {
        f184gi_config cfg{device, 0u, hbm_budget};
        status_ = f184gi_create(&cfg, &ctx_);
        if (status_ == F184GI_OK) status_ = f184gi_grid_create(ctx_, &desc, &grid_);
    }
    ~CVoxelGI() {
        for (auto& kv : cache_) {
            cudaFree(kv.second.xyz);
            cudaFree(kv.second.albedo);
        }
        cudaFree(world_);
        cudaFree(albedo_);
        if (ctx_) f184gi_destroy(ctx_);
    }
    CVoxelGI(const CVoxelGI&) = delete;
    CVoxelGI& operator=(const CVoxelGI&) = delete;

    int Status() const { return status_; }
    f184gi_ctx* Context() const { return ctx_; }
    uint32_t Grid() const { return grid_; }

    // Voxelize the visible (model matrix, primitive) pairs with the sun's injected light.
    int RenderList(const std::vector<GIMatrix3x4>& modelMats, const std::vector<const GIPrimitive*>& primitives,
                   const f184gi_light& sun, const f184gi_bounds* bounds, cudaStream_t stream = nullptr) {
        if (status_ != F184GI_OK) return status_;
        if (modelMats.size() != primitives.size()) return F184GI_ERR_INVALID;
        uint64_t total = 0;
        for (const GIPrimitive* p : primitives) total += p ? p->ntris : 0;
        if (total == 0) return F184GI_ERR_INVALID;
        int rc = Reserve(total);
        if (rc) return rc;
        uint64_t off = 0;
        for (size_t i = 0; i < primitives.size(); ++i) {
            const GIPrimitive* p = primitives[i];
            if (!p || p->ntris == 0) continue;
            const Resident* r = nullptr;
            if ((rc = Upload(p, stream, &r))) return rc;
            rc = f184gi_transform(ctx_, r->xyz, p->ntris, modelMats[i].m, world_ + off * 9, stream);
            if (rc) return rc;
            if (cudaMemcpyAsync(albedo_ + off, r->albedo, p->ntris * 4, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
                return F184GI_ERR_CUDA;
            off += p->ntris;
        }
        return f184gi_voxelize(ctx_, grid_, world_, albedo_, total, bounds, &sun, nullptr, 0, stream);
    }

    int BuildMips(cudaStream_t stream = nullptr) {
        if (status_ != F184GI_OK) return status_;
        return f184gi_mip(ctx_, grid_, 0, 0, stream);
    }

    int TraceViews(const f184gi_view* views, uint32_t nviews, const f184gi_cone_params* params = nullptr,
                   cudaStream_t stream = nullptr) {
        if (status_ != F184GI_OK) return status_;
        return f184gi_trace(ctx_, grid_, views, nviews, params, stream);
    }

    // Drop the device copy of a primitive whose geometry changed or that was destroyed.
    void Forget(const GIPrimitive* p) {
        auto it = cache_.find(p);
        if (it == cache_.end()) return;
        cudaFree(it->second.xyz);
        cudaFree(it->second.albedo);
        cache_.erase(it);
    }

private:
    struct Resident {
        float* xyz = nullptr;
        uint32_t* albedo = nullptr;
        uint64_t ntris = 0;
    };

    int Reserve(uint64_t ntris) {
        if (ntris <= capacity_) return F184GI_OK;
        cudaFree(world_);
        cudaFree(albedo_);
        world_ = nullptr;
        albedo_ = nullptr;
        if (cudaMalloc(&world_, ntris * 36) != cudaSuccess || cudaMalloc(&albedo_, ntris * 4) != cudaSuccess) {
            capacity_ = 0;
            return F184GI_ERR_OOM;
        }
        capacity_ = ntris;
        return F184GI_OK;
    }

    int Upload(const GIPrimitive* p, cudaStream_t stream, const Resident** out) {
        auto it = cache_.find(p);
        if (it != cache_.end() && it->second.ntris == p->ntris) {
            *out = &it->second;
            return F184GI_OK;
        }
        if (it != cache_.end()) Forget(p);
        Resident r;
        r.ntris = p->ntris;
        if (cudaMalloc(&r.xyz, p->ntris * 36) != cudaSuccess || cudaMalloc(&r.albedo, p->ntris * 4) != cudaSuccess) {
            cudaFree(r.xyz);
            return F184GI_ERR_OOM;
        }
        if (cudaMemcpyAsync(r.xyz, p->xyz, p->ntris * 36, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
            cudaMemcpyAsync(r.albedo, p->albedo, p->ntris * 4, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
            cudaFree(r.xyz);
            cudaFree(r.albedo);
            return F184GI_ERR_CUDA;
        }
        *out = &(cache_[p] = r);
        return F184GI_OK;
    }

    f184gi_ctx* ctx_ = nullptr;
    uint32_t grid_ = 0;
    int status_ = F184GI_OK;
    float* world_ = nullptr;
    uint32_t* albedo_ = nullptr;
    uint64_t capacity_ = 0;
    std::unordered_map<const GIPrimitive*, Resident> cache_;
};

}  // namespace Foreground
