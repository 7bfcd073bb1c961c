// Grid values of a union of spheres and boxes, evaluated in one pass.
//
// The served request stream describes each grid by such a union; evaluating it
// here writes the grid once (HBM-bound) instead of building it from a chain of
// tensor operations.  Point positions use the grid's own arithmetic
// (include/utils.cuh:62-80 of isoext, iso::grid_coord); each primitive's
// distance is the formula of isoext's sdf module (src/isoext/sdf.py:70-116):
// sphere |p - c| - r, box |max(q, 0)| + min(max(q), 0) with q = |p - c| - h.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "profile.cuh"

namespace {

constexpr int MAX_PRIMS = 32;

// prims: [0] = count (as a float), then count rows of 7 floats: kind (0 sphere,
// 1 box), centre x y z, radius | half-extents x y z.
__global__ void __launch_bounds__(256) sdf_union_grid(const float* __restrict__ prims, int nx, int ny, int nz,
                                                      float ax, float ay, float az, float sx, float sy, float sz,
                                                      bool fma, float* __restrict__ out) {
    __shared__ float pr[MAX_PRIMS][7];
    __shared__ int np;
    if (threadIdx.x == 0) np = min(max(int(prims[0]), 0), MAX_PRIMS);
    __syncthreads();
    for (int i = threadIdx.x; i < np * 7; i += blockDim.x) pr[i / 7][i % 7] = prims[1 + i];
    __syncthreads();
    // a warp per grid row (x, y), its lanes along z: the row's coordinates once,
    // consecutive lanes store consecutive values
    const int lane = threadIdx.x & 31;
    const long long rows = (long long)nx * ny;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < rows;
         row += nwarps) {
        const int y = int(row % ny), x = int(row / ny);
        const float px = iso::grid_coord(uint32_t(x), uint32_t(nx), ax, sx, fma);
        const float py = iso::grid_coord(uint32_t(y), uint32_t(ny), ay, sy, fma);
        float* orow = out + row * nz;
        for (int z = lane; z < nz; z += 32) {
            const float pz = iso::grid_coord(uint32_t(z), uint32_t(nz), az, sz, fma);
            float d = 3.402823466e38f;
            for (int k = 0; k < np; ++k) {
                const float dx = __fsub_rn(px, pr[k][1]), dy = __fsub_rn(py, pr[k][2]), dz = __fsub_rn(pz, pr[k][3]);
                float dk;
                if (pr[k][0] == 0.0f) {
                    dk = __fsub_rn(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                        __fmul_rn(dz, dz))),
                                   pr[k][4]);
                } else {
                    const float qx = __fsub_rn(fabsf(dx), pr[k][4]), qy = __fsub_rn(fabsf(dy), pr[k][5]),
                                qz = __fsub_rn(fabsf(dz), pr[k][6]);
                    const float ox = fmaxf(qx, 0.0f), oy = fmaxf(qy, 0.0f), oz = fmaxf(qz, 0.0f);
                    const float outside =
                        __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ox, ox), __fmul_rn(oy, oy)), __fmul_rn(oz, oz)));
                    dk = __fadd_rn(outside, fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f));
                }
                d = fminf(d, dk);
            }
            orow[z] = d;
        }
    }
}

}  // namespace

extern "C" {

// prims: DEVICE float [1 + 7 * count]: prims[0] = count (1 .. 32, as a float),
// then count rows of kind (0 sphere, 1 box), centre xyz, radius | half-extents
// xyz.  Reading the primitives from device memory lets a captured graph
// evaluate a new union after an upload.  out: device float [nx, ny, nz].  No
// counterpart in isoext (it builds grids with torch).
int iso_sdf_union_grid(const float* prims, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                       float* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 1 || ny < 1 || nz < 1 || !prims || !out || !aabb_min || !aabb_max) return iso::fail_code(ISO_ERR_ARG);
    const long long rows = (long long)nx * ny;  // a warp each, 8 per CTA
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long grid = std::max<long long>(1, std::min<long long>((rows + 7) / 8, (long long)sms * 8));
    iso::ProfScope ps("sdf_union_grid", st);
    sdf_union_grid<<<unsigned(grid), 256, 0, st>>>(prims, nx, ny, nz, aabb_min[0], aabb_min[1], aabb_min[2],
                                                   aabb_max[0] - aabb_min[0], aabb_max[1] - aabb_min[1],
                                                   aabb_max[2] - aabb_min[2], iso::arith_fma(), out);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

}  // extern "C"
