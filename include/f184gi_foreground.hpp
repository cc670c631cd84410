// f184gi_foreground.hpp -- C++ host adapter with the reference renderer's pass shape (header-only).
//
// Mirrors how CMegaPipeline::Render drives the GI passes (Foreground/Renderer/MegaPipeline.cpp:188-268):
//   RenderList(modelMats, primitives)  <- CZOnlyRenderer::RenderList + CVoxelizeRenderer::RenderList
//                                          (ZOnlyRenderer.h:21-22, VoxelizeRenderer.h:21-22): one (Matrix3x4,
//                                          primitive) pair per visible primitive, as CSceneView hands them out
//                                          (SceneView.h:29-33)
//   BuildMips()                         <- no reference counterpart (its volume has one level)
//   TraceViews(views)                   <- the lighting_indirect pass (MegaPipeline.cpp:241-268)
// Primitive geometry is uploaded once and kept on the device, keyed by the primitive's address (the reference
// caches per-primitive pipeline resources the same way, VoxelizeRenderer.h:47-49).  Errors come back as the C ABI's
// status codes (the reference returns silently; this adapter does not).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "f184gi.h"

namespace Foreground {

// Layout of tc::Matrix3x4 (Math/Matrix3x4.h): 12 floats, row-major, acting on column vectors.
struct GIMatrix3x4 {
    float m[12];
};
static_assert(sizeof(GIMatrix3x4) == 48, "tc::Matrix3x4 is 48 bytes");
static_assert(sizeof(f184gi_vec3) == 12, "tc::Vector3 is 12 bytes");
static_assert(sizeof(f184gi_bounds) == 32, "tc::BoundingBox is 32 bytes");

// Object-space triangle soup of one primitive (host memory, 9 floats per triangle) with per-triangle RGBA8 albedo.
struct GIPrimitive {
    const float* xyz;
    const uint32_t* albedo;
    uint64_t ntris;
};

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
            cudaMemcpyAsync(r.albedo, p->albedo, p->ntris * 4, cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return F184GI_ERR_CUDA;
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
