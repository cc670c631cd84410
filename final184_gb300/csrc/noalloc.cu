// noalloc.cu -- f184gi_gbuffer_static: the G-buffer raster with its scratch in a fixed device array.
//
// f184gi_gbuffer takes its scratch (the 64-bit depth/triangle key per pixel and the binned-raster records) from
// the context and grows it with cudaMalloc when a larger camera or mesh comes along.  Some callers cannot allow
// that: a render loop whose frame must not stall on the implicit device-wide synchronisation of cudaMalloc /
// cudaFree, or a process whose device memory is all handed out already (to a caching allocator, or to a
// context at its HBM budget).  This variant runs the same kernels on scratch carved from one file-scope
// __device__ array of kStaticScratchBytes, so a call allocates nothing on the device.
//
// Set-up: the first call on a device looks the array's address up (cudaGetSymbolAddress) with that device
// current.  That first call can load this file's module and so should come before any stream capture.  Each call
// makes the context's device current for its launches and restores the caller's device afterwards.
//
// Memory: the array's 48 MiB per device are not counted in f184gi_memory_used() nor in a request server's HBM
// budget.  They are reserved when this file's module loads on a device: at the first f184gi_gbuffer_static call
// under CUDA's default lazy module loading, at start-up of every device under CUDA_MODULE_LOADING=EAGER.
//
// Sharing: every call on a device uses the same array, which keeps the last call's contents.  The raster clears
// the counters it needs (the per-tile counts and fills, the overflow and big-record counts) on the call's
// stream, and writes every key it later reads, so calls issued one after another on one stream are correct.
// Calls that overlap on the GPU (other streams, other host threads, other contexts on the same device) race on
// the array and give undefined results.
#include <mutex>

#include "gi_internal.h"

namespace f184 {
namespace {

// Limits: at most kStaticMaxTris triangles and kStaticMaxPixels pixels (1920x1080 fits) per call.  The array
// holds the keys of kStaticMaxPixels pixels plus the raster scratch of kStaticMaxTris triangles (about 110
// bytes a triangle) with room to spare.
constexpr uint64_t kStaticMaxTris = 262144;
constexpr uint64_t kStaticMaxPixels = 2097152;
constexpr size_t kStaticScratchBytes = size_t(48) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_gbuffer_scratch[kStaticScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Once per device, with that device current (the caller makes it so): the array's device address.
int static_scratch(int device, void** ptr) {
    if (device < 0 || device >= kMaxDevices) return fail(F184GI_ERR_INVALID, "gbuffer_static: device out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_gbuffer_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "gbuffer_static: cudaGetSymbolAddress");
        g_scratch_ptr[device] = p;
    }
    *ptr = g_scratch_ptr[device];
    return F184GI_OK;
}

// The context's device current for the duration of a call, the caller's device restored at the end.
struct DeviceScope {
    int prev = -1;
    bool switched = false;
    int enter(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return cuda_fail(e, "gbuffer_static: cudaGetDevice");
        if (prev != device) {
            if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(e, "gbuffer_static: cudaSetDevice");
            switched = true;
        }
        return F184GI_OK;
    }
    ~DeviceScope() {
        if (switched) cudaSetDevice(prev);
    }
};

}  // namespace
}  // namespace f184

using namespace f184;

extern "C" int f184gi_gbuffer_static(f184gi_ctx* c, const float* tri, const float* rough, uint64_t ntris,
                                     const f184gi_view* view, uint32_t* tri_id_out, void* stream) {
    if (!c || !view || !tri || !rough) return fail(F184GI_ERR_INVALID, "gbuffer_static: null argument");
    if (!view->depth || !view->normal || !view->roughness)
        return fail(F184GI_ERR_INVALID, "gbuffer_static: null G-buffer planes");
    if (view->width == 0 || view->height == 0 || view->width > kMaxRasterSide || view->height > kMaxRasterSide)
        return fail(F184GI_ERR_INVALID,
                    "gbuffer_static: view sides must be 1.." + std::to_string(kMaxRasterSide) + " pixels");
    const uint64_t npix = uint64_t(view->width) * view->height;
    if (ntris > kStaticMaxTris)
        return fail(F184GI_ERR_INVALID, "gbuffer_static: " + std::to_string(ntris) + " triangles exceed the limit of " +
                                            std::to_string(kStaticMaxTris) + " (use f184gi_gbuffer)");
    if (npix > kStaticMaxPixels)
        return fail(F184GI_ERR_INVALID, "gbuffer_static: " + std::to_string(npix) + " pixels exceed the limit of " +
                                            std::to_string(kStaticMaxPixels) + " (use f184gi_gbuffer)");
    const size_t key_bytes = (npix * 8 + 255) & ~size_t(255);
    const size_t raster_bytes = raster_scratch_bytes(ntris, view->width, view->height);
    if (key_bytes + raster_bytes > kStaticScratchBytes)
        return fail(F184GI_ERR_INVALID, "gbuffer_static: the call needs " + std::to_string(key_bytes + raster_bytes) +
                                            " bytes of scratch, more than the " +
                                            std::to_string(kStaticScratchBytes) + " of the static array");
    double V[16], IV[16];
    for (int k = 0; k < 16; ++k) V[k] = view->view[k];
    if (!invert4(V, IV)) return fail(F184GI_ERR_INVALID, "gbuffer_static: singular view matrix");
    const float eye[3] = {float(IV[3]), float(IV[7]), float(IV[11])};
    int device = 0;
    uint32_t* d_status = nullptr;
    int rc = ctx_internal(c, &device, &d_status);
    if (rc) return rc;
    DeviceScope scope;  // the array's address and the launches belong to the context's device
    if ((rc = scope.enter(device))) return rc;
    void* base = nullptr;
    if ((rc = static_scratch(device, &base))) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    RasterJob rj{};
    rj.tri = tri;
    rj.ntris = ntris;
    view_clip_matrix(view, rj.M);  // compiled without FMA contraction, like f184gi_gbuffer's own product
    rj.d_M = nullptr;
    rj.width = view->width;
    rj.height = view->height;
    rj.keys = static_cast<unsigned long long*>(base);
    if ((rc = raster_launch(rj, static_cast<char*>(base) + key_bytes, raster_bytes, d_status, s))) return rc;
    return gbuffer_resolve_launch(rj.keys, view->width, view->height, tri, rough, view->view, eye,
                                  const_cast<float*>(view->depth), const_cast<uint32_t*>(view->normal),
                                  const_cast<uint16_t*>(view->roughness), tri_id_out, s);
}
