// iso_mc_dense_noalloc: dense marching cubes whose workspace is a fixed array
// compiled into the library, so the call needs no memory from its caller.
//
// Some callers cannot provide a workspace. A host written in C or another
// language may hold only a stream, with no device allocator. A caller may run a
// per-frame loop where it must not call cudaMalloc or cudaFree, because cudaFree
// synchronises the whole device and either call can fail partway through a
// frame. Such callers use this entry point. It runs iso_mc_dense unchanged, and
// the workspace is `g_scratch` below.
//
// Rules for callers (also stated in include/isoext_gb300.h):
//   - The scratch holds kScratchBytes (32 MiB) per device. A grid and output
//     capacities that need more are rejected with ISO_ERR_WORKSPACE before
//     anything is queued.
//   - The first call on a device does set-up. With that device current, it
//     looks up the scratch's device address (cudaGetSymbolAddress). That can
//     load the module holding the array. Make this first call before any stream
//     capture. Later calls reuse the address.
//   - All calls on a device share one scratch. Calls that overlap on the
//     device, on different streams or from different host threads without
//     ordering between them, race on it. Order them on one stream, or with
//     events.
//   - Each call clears, on its stream, the parts that must start at zero
//     (per-block tile sums and staging counters; mc_launch does this). Every
//     other byte a call reads, the same call wrote first.
#include <cstddef>
#include <cstdio>
#include <mutex>

#include <cuda_runtime.h>

#include "common.cuh"

namespace iso {
void set_last_error(const char* msg);  // capi.cu
}

extern "C" size_t iso_mc_dense_workspace_size(int nx, int ny, int nz, long long vertex_capacity,
                                              long long face_capacity);
extern "C" int iso_mc_dense(const float* values, int nx, int ny, int nz, const float* aabb_min,
                            const float* aabb_max, float level, int method, float* vertices,
                            long long vertex_capacity, int* faces, long long face_capacity, void* workspace,
                            size_t workspace_bytes, long long* counts, int* status, void* stream);

namespace {

// Must equal ISO_MC_NOALLOC_SCRATCH_BYTES in include/isoext_gb300.h.
constexpr size_t kScratchBytes = size_t(32) << 20;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        iso::set_last_error("iso_mc_dense_noalloc: cudaGetDevice failed");
        return ISO_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        iso::set_last_error("iso_mc_dense_noalloc: device ordinal above 63");
        return ISO_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "iso_mc_dense_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(e));
            iso::set_last_error(msg);
            return ISO_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return ISO_OK;
}

}  // namespace

extern "C" int iso_mc_dense_noalloc(const float* values, int nx, int ny, int nz, const float* aabb_min,
                                    const float* aabb_max, float level, int method, float* vertices,
                                    long long vertex_capacity, int* faces, long long face_capacity,
                                    long long* counts, int* status, void* stream) {
    const size_t need = iso_mc_dense_workspace_size(nx, ny, nz, vertex_capacity, face_capacity);
    if (need > kScratchBytes) {
        char msg[320];
        std::snprintf(msg, sizeof msg,
                      "iso_mc_dense_noalloc: grid %dx%dx%d with capacities %lld vertices / %lld faces "
                      "needs %zu bytes of scratch; the fixed scratch holds %zu bytes. Use iso_mc_dense "
                      "with a caller workspace.",
                      nx, ny, nz, vertex_capacity, face_capacity, need, kScratchBytes);
        iso::set_last_error(msg);
        return ISO_ERR_WORKSPACE;
    }
    void* scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    return iso_mc_dense(values, nx, ny, nz, aabb_min, aabb_max, level, method, vertices, vertex_capacity,
                        faces, face_capacity, scratch, kScratchBytes, counts, status, stream);
}
