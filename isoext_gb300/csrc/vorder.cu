// isoext's vertex order: welded vertices sorted by position, lexicographically
// in (x, y, z), with the faces renumbered (src/utils.cu:32-59 sorts the
// triangle soup with float3_less_pred and takes unique positions; the faces'
// order does not change).  The extraction kernels here number vertices by grid
// edge or by cell instead; this pass gives the reference's numbering on
// request.
//
// Two stable radix sorts (CUB) of order-preserving integer keys: by z first,
// then by (x, y); a stable sort on the major key after one on the minor key
// orders lexicographically.
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "profile.cuh"

namespace {

// Unsigned key whose order is the float's order (-0 and +0 equal, as the
// reference's float comparison has them).
__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t u = __float_as_uint(f == 0.0f ? 0.0f : f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void vo_keys_z(const float* __restrict__ v, long long V, uint32_t* __restrict__ kz,
                          uint32_t* __restrict__ idx) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    kz[i] = fkey(v[3 * i + 2]);
    idx[i] = uint32_t(i);
}

__global__ void vo_keys_xy(const float* __restrict__ v, long long V, const uint32_t* __restrict__ idx,
                           unsigned long long* __restrict__ kxy) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const uint32_t j = idx[i];
    kxy[i] = ((unsigned long long)fkey(v[3 * j]) << 32) | fkey(v[3 * j + 1]);
}

// perm[i] = the old index of new vertex i: gather positions, invert.
__global__ void vo_gather(const float* __restrict__ v, long long V, const uint32_t* __restrict__ perm,
                          float* __restrict__ vtmp, uint32_t* __restrict__ newidx) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const uint32_t j = perm[i];
    vtmp[3 * i] = v[3 * j];
    vtmp[3 * i + 1] = v[3 * j + 1];
    vtmp[3 * i + 2] = v[3 * j + 2];
    newidx[j] = uint32_t(i);
}

__global__ void vo_copy_back(const float* __restrict__ vtmp, long long n, float* __restrict__ v) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = vtmp[i];
}

__global__ void vo_remap(int32_t* __restrict__ f, long long n, const uint32_t* __restrict__ newidx) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f[i] = int32_t(newidx[f[i]]);
}

struct VoWs {
    uint32_t *kz, *kz2, *i0, *i1, *newidx;
    unsigned long long *kxy, *kxy2;
    float* vtmp;
    void* temp;
    size_t temp_bytes, total;
};

size_t cub_temp(long long V) {
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, int(V));
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, int(V));
    return a > b ? a : b;
}

VoWs vo_carve(void* ws, long long V) {
    VoWs w{};
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = ws ? b + o : nullptr;
        o = (o + (bytes ? bytes : 1) + 255) & ~size_t(255);
        return p;
    };
    w.kz = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.kz2 = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.i0 = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.i1 = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.newidx = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.kxy = reinterpret_cast<unsigned long long*>(take(size_t(V) * 8));
    w.kxy2 = reinterpret_cast<unsigned long long*>(take(size_t(V) * 8));
    w.vtmp = reinterpret_cast<float*>(take(size_t(V) * 12));
    w.temp_bytes = cub_temp(V);
    w.temp = take(w.temp_bytes);
    w.total = o + 256;
    return w;
}

unsigned blocks(long long n) { return unsigned((n + 255) / 256); }

}  // namespace

extern "C" {

size_t iso_sort_vertices_workspace_size(long long num_vertices) {
    if (num_vertices < 0 || num_vertices > 0x7fffffffll) return 0;
    return vo_carve(nullptr, num_vertices).total;
}

// Renumbers a welded mesh in isoext's vertex order, in place: vertices
// (device float [V, 3], distinct positions) sorted lexicographically by
// (x, y, z), faces (device int32 [F, 3]) renumbered to match.
int iso_sort_vertices(float* vertices, long long num_vertices, int* faces, long long num_faces, void* workspace,
                      size_t workspace_bytes, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const long long V = num_vertices, F = num_faces;
    if (V < 0 || F < 0 || V > 0x7fffffffll || (V && !vertices) || (F && !faces)) return iso::fail_code(ISO_ERR_ARG);
    if (V <= 1) return ISO_OK;
    if (workspace_bytes < iso_sort_vertices_workspace_size(V) || !workspace) return iso::fail_code(ISO_ERR_WORKSPACE);
    VoWs w = vo_carve(workspace, V);
    iso::ProfScope ps("vertex_order", st, 7);
    vo_keys_z<<<blocks(V), 256, 0, st>>>(vertices, V, w.kz, w.i0);
    size_t tb = w.temp_bytes;
    if (cub::DeviceRadixSort::SortPairs(w.temp, tb, w.kz, w.kz2, w.i0, w.i1, int(V), 0, 32, st) != cudaSuccess)
        return iso::fail_code(ISO_ERR_CUDA);
    vo_keys_xy<<<blocks(V), 256, 0, st>>>(vertices, V, w.i1, w.kxy);
    tb = w.temp_bytes;
    if (cub::DeviceRadixSort::SortPairs(w.temp, tb, w.kxy, w.kxy2, w.i1, w.i0, int(V), 0, 64, st) != cudaSuccess)
        return iso::fail_code(ISO_ERR_CUDA);
    vo_gather<<<blocks(V), 256, 0, st>>>(vertices, V, w.i0, w.vtmp, w.newidx);
    vo_copy_back<<<blocks(3 * V), 256, 0, st>>>(w.vtmp, 3 * V, vertices);
    if (F) vo_remap<<<blocks(3 * F), 256, 0, st>>>(faces, 3 * F, w.newidx);
    return cudaGetLastError() == cudaSuccess ? ISO_OK : iso::fail_code(ISO_ERR_CUDA);
}

}  // extern "C"
