// C ABI of libisoext_gb300.so (declared in include/isoext_gb300.h).
//
// Every entry point takes raw device pointers, sizes and a cudaStream_t, runs
// asynchronously on that stream, and returns an IsoStatus for argument / launch
// errors.  Errors found on the device (bounded waits that ran out, output
// capacity exceeded) are written to the caller's device status word.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "common.cuh"
#include "mc_dense.cuh"

namespace {
thread_local std::string g_err;

int fail(int code, const char* msg) {
    g_err = msg;
    return code;
}

bool grid_ok(int nx, int ny, int nz) {
    if (nx < 0 || ny < 0 || nz < 0) return false;
    return (long long)nx * ny * nz <= 0x7fffffffll;
}
}  // namespace

namespace iso {
// Message iso_last_error returns on this thread (for entry points in other files).
void set_last_error(const char* msg) { g_err = msg; }

int fail_code(int code) {
    switch (code) {
        case ISO_ERR_ARG: g_err = "invalid argument"; break;
        case ISO_ERR_CUDA: g_err = std::string("CUDA call failed: ") + cudaGetErrorString(cudaPeekAtLastError()); break;
        case ISO_ERR_TIMEOUT: g_err = "a bounded wait ran out"; break;
        case ISO_ERR_LOOKUP: g_err = "lookup failed"; break;
        case ISO_ERR_WORKSPACE: g_err = "workspace too small"; break;
        case ISO_ERR_OVERFLOW: g_err = "output capacity exceeded"; break;
        default: g_err = "error " + std::to_string(code); break;
    }
    return code;
}

// Tunables: sign-pass CTAs per SM (MC and DC sign bitmaps), threads per block of
// the per-active-cell DC kernels, threads per block of the MC count kernel.
std::atomic<int> g_tune[TUNE_KEYS] = {{32}, {128}, {256}};
int tune_get(int key) { return key >= 0 && key < TUNE_KEYS ? g_tune[key].load(std::memory_order_relaxed) : 0; }

// Arithmetic reading of the reference's expressions (common.cuh): 1 = its CUDA
// build's fused multiply-adds (the default), 0 = its host build.
std::atomic<int> g_arith{1};
bool arith_fma() { return g_arith.load(std::memory_order_relaxed) != 0; }
}  // namespace iso

namespace {
// Coordinates of the n points of one grid axis (include/utils.cuh:62-80).
__global__ void axis_coords_kernel(float* out, int n, float amin, float size, bool fma) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = iso::grid_coord(uint32_t(i), uint32_t(n), amin, size, fma);
}
}  // namespace

extern "C" {

const char* iso_last_error(void) { return g_err.c_str(); }

int iso_abi_version(void) { return 2; }

int iso_set_arith(int mode) {
    if (mode != 0 && mode != 1) return fail(ISO_ERR_ARG, "iso_set_arith: mode must be 0 (host build) or 1 (CUDA build)");
    iso::g_arith.store(mode, std::memory_order_relaxed);
    return ISO_OK;
}

int iso_get_arith(void) { return iso::g_arith.load(std::memory_order_relaxed); }

int iso_axis_coords(float* out, int n, float amin, float amax, void* stream) {
    if (n < 0 || (n > 0 && !out)) return fail(ISO_ERR_ARG, "iso_axis_coords: bad arguments");
    if (n == 0) return ISO_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    axis_coords_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(out, n, amin, amax - amin, iso::arith_fma());
    return cudaGetLastError() == cudaSuccess ? ISO_OK : fail(ISO_ERR_CUDA, "iso_axis_coords: launch failed");
}

int iso_mc_set_config(int threads) {
    if (mc_set_block(threads)) return fail(ISO_ERR_ARG, "iso_mc_set_config: threads must be 128 or 256");
    return ISO_OK;
}

int iso_mc_get_config(int* threads) {
    if (threads) *threads = mc_get_block();
    return ISO_OK;
}

int iso_tune_set(const char* key, int value) {
    if (!key) return fail(ISO_ERR_ARG, "iso_tune_set: key is null");
    if (!strcmp(key, "mc.emit_threads")) {
        if (mc_set_block(value)) return fail(ISO_ERR_ARG, "mc.emit_threads must be 128 or 256");
        return ISO_OK;
    }
    if (!strcmp(key, "mc.sign_ctas_per_sm")) {
        if (value < 1 || value > 64) return fail(ISO_ERR_ARG, "mc.sign_ctas_per_sm must be 1 .. 64");
        iso::g_tune[iso::TUNE_MC_SIGN_CTAS] = value;
        return ISO_OK;
    }
    if (!strcmp(key, "dc.cell_threads")) {
        if (value != 64 && value != 128 && value != 256) return fail(ISO_ERR_ARG, "dc.cell_threads must be 64, 128 or 256");
        iso::g_tune[iso::TUNE_DC_CELL_THREADS] = value;
        return ISO_OK;
    }
    if (!strcmp(key, "mc.count_threads")) {
        if (value != 128 && value != 256) return fail(ISO_ERR_ARG, "mc.count_threads must be 128 or 256");
        iso::g_tune[iso::TUNE_MC_COUNT_THREADS] = value;
        return ISO_OK;
    }
    return fail(ISO_ERR_ARG, "iso_tune_set: unknown key");
}

int iso_tune_get(const char* key, int* value) {
    if (!key || !value) return fail(ISO_ERR_ARG, "iso_tune_get: null argument");
    if (!strcmp(key, "mc.emit_threads")) *value = mc_get_block();
    else if (!strcmp(key, "mc.sign_ctas_per_sm")) *value = iso::tune_get(iso::TUNE_MC_SIGN_CTAS);
    else if (!strcmp(key, "dc.cell_threads")) *value = iso::tune_get(iso::TUNE_DC_CELL_THREADS);
    else if (!strcmp(key, "mc.count_threads")) *value = iso::tune_get(iso::TUNE_MC_COUNT_THREADS);
    else return fail(ISO_ERR_ARG, "iso_tune_get: unknown key");
    return ISO_OK;
}

size_t iso_mc_dense_workspace_size(int nx, int ny, int nz, long long vertex_capacity,
                                   long long face_capacity) {
    if (!grid_ok(nx, ny, nz) || nx < 2 || ny < 2 || nz < 2) return 256;
    if (vertex_capacity < 0 || face_capacity < 0) return 0;
    return mc_workspace_bytes(nx, ny, nz, vertex_capacity, face_capacity);
}

}  // extern "C"

namespace {

int mc_dense_impl(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                  float level, int method, float* vertices, long long vertex_capacity, int* faces,
                  long long face_capacity, void* workspace, size_t workspace_bytes, long long* counts,
                  int* status, long long* vertex_edges, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!grid_ok(nx, ny, nz))
        return fail(ISO_ERR_ARG, "Number of points exceeds maximum value 2147483647 (max int)");
    if (method != 0 && method != 1) return fail(ISO_ERR_ARG, "method must be 0 (nagae) or 1 (lorensen)");
    if (!counts || !status || !aabb_min || !aabb_max)
        return fail(ISO_ERR_ARG, "counts, status and the bounding box are required");
    if (vertex_capacity < 0 || face_capacity < 0) return fail(ISO_ERR_ARG, "negative capacity");
    if (nx < 2 || ny < 2 || nz < 2) {
        // no cells: empty mesh
        if (cudaMemsetAsync(counts, 0, 2 * sizeof(long long), st) != cudaSuccess)
            return fail(ISO_ERR_CUDA, "cudaMemsetAsync failed");
        return ISO_OK;
    }
    if (!values) return fail(ISO_ERR_ARG, "values is null");
    if (reinterpret_cast<uintptr_t>(values) & 15u)
        return fail(ISO_ERR_ARG, "values must be 16-byte aligned");
    if ((vertex_capacity && !vertices) || (face_capacity && !faces))
        return fail(ISO_ERR_ARG, "output buffers are null");
    McParams p{};
    p.vals = values;
    p.nx = nx; p.ny = ny; p.nz = nz;
    for (int i = 0; i < 3; ++i) {
        p.amin[i] = aabb_min[i];
        p.asize[i] = aabb_max[i] - aabb_min[i];  // FP32, as aabb_max - aabb_min in the reference
    }
    p.level = level;
    p.method = method;
    p.status = status;
    p.vout = vertices;
    p.fout = faces;
    p.capV = vertex_capacity;
    p.capF = face_capacity;
    p.counts = counts;
    p.vedge = vertex_edges;
    int rc = mc_launch(p, workspace, workspace_bytes, st);
    if (rc == ISO_ERR_WORKSPACE) return fail(rc, "workspace too small");
    if (rc) {
        g_err = std::string("launch failed: ") + cudaGetErrorString(cudaGetLastError());
        return rc;
    }
    return ISO_OK;
}

}  // namespace

extern "C" {

int iso_mc_dense(const float* values, int nx, int ny, int nz, const float* aabb_min,
                 const float* aabb_max, float level, int method, float* vertices,
                 long long vertex_capacity, int* faces, long long face_capacity, void* workspace,
                 size_t workspace_bytes, long long* counts, int* status, void* stream) {
    return mc_dense_impl(values, nx, ny, nz, aabb_min, aabb_max, level, method, vertices, vertex_capacity, faces,
                         face_capacity, workspace, workspace_bytes, counts, status, nullptr, stream);
}

int iso_mc_dense_edges(const float* values, int nx, int ny, int nz, const float* aabb_min,
                       const float* aabb_max, float level, int method, float* vertices,
                       long long vertex_capacity, int* faces, long long face_capacity, void* workspace,
                       size_t workspace_bytes, long long* counts, int* status, long long* vertex_edges,
                       void* stream) {
    if (!vertex_edges && vertex_capacity) return fail(ISO_ERR_ARG, "vertex_edges is null");
    return mc_dense_impl(values, nx, ny, nz, aabb_min, aabb_max, level, method, vertices, vertex_capacity, faces,
                         face_capacity, workspace, workspace_bytes, counts, status, vertex_edges, stream);
}

}  // extern "C"
