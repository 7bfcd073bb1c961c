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
//   - Every call looks up the scratch's device address (cudaGetSymbolAddress)
//     in the CUDA context current on the calling thread, so a context made
//     after a cudaDeviceReset, or a caller's own driver context, gets its own
//     copy of the array. The first lookup in a context can load the module
//     holding the array: make that first call before any stream capture.
//   - All calls in one context share one scratch. Calls that overlap on the
//     device, on different streams or from different host threads without
//     ordering between them, race on it. Order them on one stream, or with
//     events.
//   - Each call clears, on its stream, the parts that must start at zero: the
//     sign pass (mc_signs) zeroes the counters, the scan's look-back states and
//     the merge hash before the later kernels read them. Every other byte a call
//     reads, the same call wrote first.
#include <cstddef>
#include <cstdio>

#include <cuda_runtime.h>

#include "isoext_gb300.h"

namespace iso {
void set_last_error(const char* msg);  // capi.cu
}

namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;
static_assert(kScratchBytes == ISO_MC_NOALLOC_SCRATCH_BYTES, "the header states the scratch size");

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The scratch's address in the context current on this thread.  Looked up on
// every call rather than cached per device: a cached address would outlive a
// cudaDeviceReset, and would be another context's memory for a caller that
// makes its own driver context current.
int scratch_address(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "iso_mc_dense_noalloc: cudaGetSymbolAddress failed: %s",
                      cudaGetErrorString(e));
        iso::set_last_error(msg);
        return ISO_ERR_CUDA;
    }
    *out = p;
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
