// TEST INFRASTRUCTURE ONLY: isoext's device arithmetic as its CUDA build
// computes it, to pin the library's default ("nvcc") reading bit for bit.
//
// isoext's GPU build compiles its expressions with nvcc's default flags, and
// nvcc's default -fmad=true fuses multiply-adds wherever it chooses.  Which
// product it fuses depends on the shape of the source, so this file restates
// the reference's device expressions in the same shape -- float3 operators,
// the lerp template, the trilinear helper called six times per crossing -- and
// is compiled by tests/test_nvcc_parity_gpu.py with default flags (no -fmad,
// no rounding intrinsics), as the reference's CMake build does
// (CMakeLists.txt sets only --extended-lambda).  The library's kernels and the
// oracle spell each fused operation out explicitly (isoext_gb300/csrc/common.cuh,
// oracle/iso_oracle.c), so a match here shows that the explicit forms are the
// ones nvcc picks.
//
// Restated expressions (paths inside the isoext project):
//   grid point position   include/utils.cuh:62-80    (get_vtx_pos_op)
//   float3 operators      include/math.cuh:22-75
//   lerp                  include/math.cuh:77-81
//   crossing point        src/its.cu:60-88, src/mc/nagae.cu:47-57 (same lerp)
//   normal stencil        src/its.cu:170-268         (trilinear_interp, compute_normals_op)
//   norm / dot            include/math.cuh:83-96
//   QEF accumulation      src/dc.cu:14-65            (get_qef_op)
#include <cstdint>
#include <cuda_runtime.h>

using uint = unsigned int;

namespace {

__host__ __device__ inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline float3 operator*(float3 a, float b) { return make_float3(a.x * b, a.y * b, a.z * b); }
__host__ __device__ inline float3 operator*(float a, float3 b) { return make_float3(a * b.x, a * b.y, a * b.z); }
__host__ __device__ inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ inline float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
__host__ __device__ inline float3 operator/(float3 a, float b) { return make_float3(a.x / b, a.y / b, a.z / b); }

template <typename T>
__host__ __device__ T lerp(float t, T a, T b) {
    return (1 - t) * a + t * b;
}

__host__ __device__ inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float norm(float3 a) { return sqrt(dot(a, a)); }

// Point position from its linear id.
__device__ float3 point_position(uint idx, uint3 res, float3 aabb_min, float3 aabb_size) {
    float3 pos;
    pos.z = (idx % res.z) / (float)(res.z - 1);
    idx /= res.z;
    pos.y = (idx % res.y) / (float)(res.y - 1);
    pos.x = (idx / res.y) / (float)(res.x - 1);
    pos = aabb_min + pos * aabb_size;
    return pos;
}

__global__ void k_points(uint n, uint3 res, float3 aabb_min, float3 aabb_size, float3* out) {
    const uint i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = point_position(i, res, aabb_min, aabb_size);
}

// Point ids of the 8 corners of cell c, corner k = 4x + 2y + z.
__device__ void cell_corners(uint c, uint3 res, uint* ids) {
    const uint z = c % (res.z - 1), r = c / (res.z - 1);
    const uint y = r % (res.y - 1), x = r / (res.y - 1);
    const uint base = (x * res.y + y) * res.z + z, yz = res.y * res.z;
    for (int k = 0; k < 8; ++k) ids[k] = base + (k >> 2) * yz + ((k >> 1) & 1) * res.z + (k & 1);
}

// Crossing points of active cells, edges in ascending order, written from the
// cell's CSR offset; a cell whose crossing count disagrees with the offsets
// sets *bad.
__global__ void k_crossings(uint ncells, uint3 res, const float* values, const float3* points,
                            const int* cell_indices, const int* cell_offsets, const int* edges_table, float level,
                            float3* its_points, int* bad) {
    const uint idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncells) return;
    uint ids[8];
    cell_corners(uint(cell_indices[idx]), res, ids);
    float3 c_p[8];
    float c_v[8];
    int status = 0;
    for (uint32_t i = 0; i < 8; i++) {
        c_p[i] = points[ids[i]];
        c_v[i] = values[ids[i]];
    }
    for (int i = 0; i < 12; i++) {
        const int a = edges_table[2 * i], b = edges_table[2 * i + 1];
        if ((c_v[a] - level < 0) != (c_v[b] - level < 0)) status |= 1 << i;
    }
    int offset = cell_offsets[idx];
    for (int i = 0; i < 12; i++) {
        if (status & (1 << i)) {
            int p_0 = edges_table[i * 2];
            int p_1 = edges_table[i * 2 + 1];
            float denom = c_v[p_1] - c_v[p_0];
            float t = (denom != 0.0f) ? (level - c_v[p_0]) / denom : 0.0f;
            if (offset < cell_offsets[idx + 1]) its_points[offset] = lerp(t, c_p[p_0], c_p[p_1]);
            offset++;
        }
    }
    if (offset != cell_offsets[idx + 1]) atomicExch(bad, 1);
}

__host__ __device__ float trilinear_interp(float3 t, const float* c_v) {
    float c00 = c_v[0] * (1 - t.z) + c_v[1] * t.z;
    float c01 = c_v[2] * (1 - t.z) + c_v[3] * t.z;
    float c10 = c_v[4] * (1 - t.z) + c_v[5] * t.z;
    float c11 = c_v[6] * (1 - t.z) + c_v[7] * t.z;
    float c0 = c00 * (1 - t.y) + c01 * t.y;
    float c1 = c10 * (1 - t.y) + c11 * t.y;
    return c0 * (1 - t.x) + c1 * t.x;
}

// Normals of the crossings of each active cell.
__global__ void k_normals(uint ncells, uint3 res, const float* values, const float3* grid_points,
                          const int* cell_indices, const int* cell_offsets, const float3* its_points,
                          float3* normals) {
    const uint cell_idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell_idx >= ncells) return;
    uint offset = cell_offsets[cell_idx];
    uint next_offset = cell_offsets[cell_idx + 1];
    uint ids[8];
    cell_corners(uint(cell_indices[cell_idx]), res, ids);
    float c_v[8];
    float3 c_p[8];
    for (uint i = 0; i < 8; i++) {
        c_p[i] = grid_points[ids[i]];
        c_v[i] = values[ids[i]];
    }
    float3 cell_min = c_p[0];
    float3 cell_size = c_p[7] - c_p[0];
    for (uint i = offset; i < next_offset; i++) {
        float3 p = its_points[i];
        float3 t = (p - cell_min) / cell_size;
        t.x = fmaxf(0.01f, fminf(0.99f, t.x));
        t.y = fmaxf(0.01f, fminf(0.99f, t.y));
        t.z = fmaxf(0.01f, fminf(0.99f, t.z));
        float eps = 0.02f;
        float3 t_px = make_float3(fminf(t.x + eps, 0.99f), t.y, t.z);
        float3 t_mx = make_float3(fmaxf(t.x - eps, 0.01f), t.y, t.z);
        float3 t_py = make_float3(t.x, fminf(t.y + eps, 0.99f), t.z);
        float3 t_my = make_float3(t.x, fmaxf(t.y - eps, 0.01f), t.z);
        float3 t_pz = make_float3(t.x, t.y, fminf(t.z + eps, 0.99f));
        float3 t_mz = make_float3(t.x, t.y, fmaxf(t.z - eps, 0.01f));
        float dfdx = (trilinear_interp(t_px, c_v) - trilinear_interp(t_mx, c_v)) / ((t_px.x - t_mx.x) * cell_size.x);
        float dfdy = (trilinear_interp(t_py, c_v) - trilinear_interp(t_my, c_v)) / ((t_py.y - t_my.y) * cell_size.y);
        float dfdz = (trilinear_interp(t_pz, c_v) - trilinear_interp(t_mz, c_v)) / ((t_pz.z - t_mz.z) * cell_size.z);
        float3 grad = make_float3(dfdx, dfdy, dfdz);
        float grad_len = norm(grad);
        float3 n;
        if (grad_len > 1e-8f) {
            n = grad / grad_len;
        } else {
            n = make_float3(0.0f, 0.0f, 1.0f);
        }
        normals[i] = n;
    }
}

// QEF of each active cell: ATA [ncells, 9] and ATb [ncells, 3], zeroed by the
// caller and accumulated in place.
__global__ void k_qef(uint ncells, const float3* its_points, const float3* its_normals, const int* its_cell_offsets,
                      float reg, float* ATA, float* ATb) {
    const uint idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncells) return;
    uint ATA_offset = idx * 9;
    uint ATb_offset = idx * 3;
    float3 p_avg = make_float3(0.0f, 0.0f, 0.0f);
    for (uint i = its_cell_offsets[idx]; i < uint(its_cell_offsets[idx + 1]); i++) {
        float3 n = its_normals[i];
        float3 p = its_points[i];
        float3 nnp = n * dot(n, p);
        p_avg = p_avg + p;
        ATA[ATA_offset + 0] += n.x * n.x;
        ATA[ATA_offset + 1] += n.x * n.y;
        ATA[ATA_offset + 2] += n.x * n.z;
        ATA[ATA_offset + 3] += n.y * n.x;
        ATA[ATA_offset + 4] += n.y * n.y;
        ATA[ATA_offset + 5] += n.y * n.z;
        ATA[ATA_offset + 6] += n.z * n.x;
        ATA[ATA_offset + 7] += n.z * n.y;
        ATA[ATA_offset + 8] += n.z * n.z;
        ATb[ATb_offset + 0] += nnp.x;
        ATb[ATb_offset + 1] += nnp.y;
        ATb[ATb_offset + 2] += nnp.z;
    }
    p_avg = p_avg / (uint(its_cell_offsets[idx + 1]) - uint(its_cell_offsets[idx]));
    ATA[ATA_offset + 0] += reg;
    ATA[ATA_offset + 4] += reg;
    ATA[ATA_offset + 8] += reg;
    ATb[ATb_offset + 0] += reg * p_avg.x;
    ATb[ATb_offset + 1] += reg * p_avg.y;
    ATb[ATb_offset + 2] += reg * p_avg.z;
}

unsigned blocks(uint n) { return (n + 255) / 256; }

}  // namespace

extern "C" {

// All pointers are device pointers; aabb_* are host float[3].  Each call
// returns the launch's cudaError_t.
int nx_points(int nx, int ny, int nz, const float* aabb_min, const float* aabb_max, float* out, void* stream) {
    const uint3 res = make_uint3(uint(nx), uint(ny), uint(nz));
    const float3 lo = make_float3(aabb_min[0], aabb_min[1], aabb_min[2]);
    const float3 size = make_float3(aabb_max[0] - aabb_min[0], aabb_max[1] - aabb_min[1], aabb_max[2] - aabb_min[2]);
    const uint n = uint(nx) * uint(ny) * uint(nz);
    k_points<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(n, res, lo, size, reinterpret_cast<float3*>(out));
    return int(cudaGetLastError());
}

int nx_crossings(int nx, int ny, int nz, const float* values, const float* points, const int* cell_indices,
                 const int* cell_offsets, int ncells, const int* edges_table, float level, float* its_points,
                 int* bad, void* stream) {
    const uint3 res = make_uint3(uint(nx), uint(ny), uint(nz));
    if (ncells > 0)
        k_crossings<<<blocks(uint(ncells)), 256, 0, (cudaStream_t)stream>>>(
            uint(ncells), res, values, reinterpret_cast<const float3*>(points), cell_indices, cell_offsets,
            edges_table, level, reinterpret_cast<float3*>(its_points), bad);
    return int(cudaGetLastError());
}

int nx_normals(int nx, int ny, int nz, const float* values, const float* points, const int* cell_indices,
               const int* cell_offsets, int ncells, const float* its_points, float* normals, void* stream) {
    const uint3 res = make_uint3(uint(nx), uint(ny), uint(nz));
    if (ncells > 0)
        k_normals<<<blocks(uint(ncells)), 256, 0, (cudaStream_t)stream>>>(
            uint(ncells), res, values, reinterpret_cast<const float3*>(points), cell_indices, cell_offsets,
            reinterpret_cast<const float3*>(its_points), reinterpret_cast<float3*>(normals));
    return int(cudaGetLastError());
}

int nx_qef(const float* its_points, const float* its_normals, const int* cell_offsets, int ncells, float reg,
           float* ata, float* atb, void* stream) {
    if (ncells > 0)
        k_qef<<<blocks(uint(ncells)), 256, 0, (cudaStream_t)stream>>>(
            uint(ncells), reinterpret_cast<const float3*>(its_points), reinterpret_cast<const float3*>(its_normals),
            cell_offsets, reg, ata, atb);
    return int(cudaGetLastError());
}

}  // extern "C"
