// adapter_main.cpp -- drives the C++ adapter (include/f184gi_foreground.hpp) the way CMegaPipeline drives its
// passes, and checks it against the plain C ABI path on the same scene.  Exit code 0 = identical results.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "f184gi_foreground.hpp"

#define CHECK(x)                                                                           \
    do {                                                                                   \
        int rc_ = (x);                                                                     \
        if (rc_ != 0) {                                                                    \
            std::fprintf(stderr, "%s failed: %d (%s)\n", #x, rc_, f184gi_last_error());   \
            return 1;                                                                      \
        }                                                                                  \
    } while (0)

int main() {
    f184gi_scene* sc = nullptr;
    CHECK(f184gi_scene_generate(184, 20000, 200, &sc));
    const uint32_t W = 320, H = 180;
    f184gi_grid_desc desc{64, 6, F184GI_FMT_F32, 0, 1024, 0};
    // adapter path: one primitive per scene object, identity model matrices
    Foreground::CVoxelGI gi(desc);
    CHECK(gi.Status());
    std::vector<Foreground::GIPrimitive> prims(sc->nobjects);
    std::vector<const Foreground::GIPrimitive*> list;
    std::vector<Foreground::GIMatrix3x4> mats;
    const Foreground::GIMatrix3x4 ident{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}};
    for (uint32_t o = 0; o < sc->nobjects; ++o) {
        prims[o] = {sc->tri_xyz + uint64_t(sc->object_first[o]) * 9, sc->albedo + sc->object_first[o], sc->object_count[o]};
        list.push_back(&prims[o]);
        mats.push_back(ident);
    }
    CHECK(gi.RenderList(mats, list, sc->light, &sc->bounds));
    CHECK(gi.BuildMips());
    // G-buffer + trace through the adapter's context
    float view[16], proj[16];
    f184gi_camera_look_at(sc->eye, sc->target, view);
    f184gi_camera_perspective(59.0f, float(W) / float(H), 0.1f, 100.0f, proj);
    float *d_tri, *d_rough, *d_depth, *d_out, *d_out2;
    uint32_t* d_normal;
    uint16_t* d_rgh;
    cudaMalloc(&d_tri, sc->ntris * 36);
    cudaMalloc(&d_rough, sc->ntris * 4);
    cudaMalloc(&d_depth, W * H * 4);
    cudaMalloc(&d_normal, W * H * 4);
    cudaMalloc(&d_rgh, W * H * 2);
    cudaMalloc(&d_out, W * H * 32);
    cudaMalloc(&d_out2, W * H * 32);
    cudaMemcpy(d_tri, sc->tri_xyz, sc->ntris * 36, cudaMemcpyHostToDevice);
    cudaMemcpy(d_rough, sc->roughness, sc->ntris * 4, cudaMemcpyHostToDevice);
    f184gi_view v{};
    std::memcpy(v.view, view, 64);
    std::memcpy(v.proj, proj, 64);
    v.width = W, v.height = H, v.depth = d_depth, v.normal = d_normal, v.roughness = d_rgh, v.out = d_out;
    v.out_format = F184GI_FMT_F32;
    CHECK(f184gi_gbuffer(gi.Context(), d_tri, d_rough, sc->ntris, &v, nullptr, nullptr));
    CHECK(gi.TraceViews(&v, 1));
    CHECK(f184gi_sync(gi.Context(), nullptr));
    // plain C ABI path on the world-space triangles
    f184gi_ctx* ctx = nullptr;
    f184gi_config cfg{0, 0, 0};
    CHECK(f184gi_create(&cfg, &ctx));
    uint32_t grid = 0;
    CHECK(f184gi_grid_create(ctx, &desc, &grid));
    uint32_t* d_alb;
    cudaMalloc(&d_alb, sc->ntris * 4);
    cudaMemcpy(d_alb, sc->albedo, sc->ntris * 4, cudaMemcpyHostToDevice);
    CHECK(f184gi_voxelize(ctx, grid, d_tri, d_alb, sc->ntris, &sc->bounds, &sc->light, nullptr, 0, nullptr));
    CHECK(f184gi_mip(ctx, grid, 0, 0, nullptr));
    f184gi_view v2 = v;
    v2.out = d_out2;
    CHECK(f184gi_trace(ctx, grid, &v2, 1, nullptr, nullptr));
    CHECK(f184gi_sync(ctx, nullptr));
    std::vector<float> a(W * H * 8), b(W * H * 8);
    cudaMemcpy(a.data(), d_out, a.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), d_out2, b.size() * 4, cudaMemcpyDeviceToHost);
    double sum = 0.0;
    for (float x : a) sum += x;
    bool same = std::memcmp(a.data(), b.data(), a.size() * 4) == 0;
    std::printf("adapter %s the C ABI path (%llu triangles in %u primitives, mean output %.6f)\n",
                same ? "matches" : "DIFFERS FROM", (unsigned long long)sc->ntris, sc->nobjects, sum / a.size());

    // view culling: the camera frustum placed in the world, the primitives outside it dropped by CullList, the
    // kept ones voxelized through the adapter and, concatenated on the host, through the C ABI: same L0 bytes
    Foreground::GIFrustum cam;
    CHECK(Foreground::GIFrustumDefine(proj, &cam));
    float world[16];
    CHECK(f184gi_mat4_inverse(view, world));  // the camera node's world transform
    Foreground::GIMatrix3x4 cam_world;
    std::memcpy(cam_world.m, world, 48);
    std::vector<Foreground::GIMatrix3x4> kept_mats;
    std::vector<const Foreground::GIPrimitive*> kept;
    Foreground::CullList(Foreground::GIFrustumTransformed(cam, cam_world), mats, list, kept_mats, kept);
    Foreground::CVoxelGI culled(desc);
    CHECK(culled.Status());
    CHECK(culled.RenderList(kept_mats, kept, sc->light, &sc->bounds));
    std::vector<float> soup;
    std::vector<uint32_t> soup_alb;
    for (const Foreground::GIPrimitive* p : kept) {
        soup.insert(soup.end(), p->xyz, p->xyz + p->ntris * 9);
        soup_alb.insert(soup_alb.end(), p->albedo, p->albedo + p->ntris);
    }
    uint64_t nkept = soup_alb.size();
    float* d_soup = nullptr;
    uint32_t* d_soup_alb = nullptr;
    cudaMalloc(&d_soup, nkept * 36);
    cudaMalloc(&d_soup_alb, nkept * 4);
    cudaMemcpy(d_soup, soup.data(), nkept * 36, cudaMemcpyHostToDevice);
    cudaMemcpy(d_soup_alb, soup_alb.data(), nkept * 4, cudaMemcpyHostToDevice);
    uint32_t grid2 = 0;
    CHECK(f184gi_grid_create(ctx, &desc, &grid2));
    CHECK(f184gi_voxelize(ctx, grid2, d_soup, d_soup_alb, nkept, &sc->bounds, &sc->light, nullptr, 0, nullptr));
    CHECK(f184gi_sync(ctx, nullptr));
    CHECK(f184gi_sync(culled.Context(), nullptr));
    const size_t nvox = size_t(desc.dim) * desc.dim * desc.dim * 4;
    std::vector<float> la(nvox), lb(nvox);
    CHECK(f184gi_grid_read_level(culled.Context(), culled.Grid(), 0, 0, la.data()));
    CHECK(f184gi_grid_read_level(ctx, grid2, 0, 0, lb.data()));
    const bool same_culled = std::memcmp(la.data(), lb.data(), nvox * 4) == 0;
    std::printf("culled adapter %s the C ABI path (%zu of %u primitives kept, %llu triangles)\n",
                same_culled ? "matches" : "DIFFERS FROM", kept.size(), sc->nobjects, (unsigned long long)nkept);
    const bool culled_some = !kept.empty() && kept.size() < sc->nobjects;
    f184gi_destroy(ctx);
    f184gi_scene_free(sc);
    return same && sum > 0.0 && same_culled && culled_some ? 0 : 2;
}
