// Dense-grid marching cubes: parameters, workspace and launch API.
//
// Layout.  Grid values are float32 [nx, ny, nz] (z fastest).  The sign bitmap
// holds bit z % 32 of word  pw = (x * ny + y) * NW + z / 32  (NW = ceil(nz / 32))
// for v(x, y, z) - level < 0.  A "point word" pw also names the 32 grid edges
// along each axis whose LOW endpoint lies in it, and the 32 cells whose lowest
// corner lies in it.
//
// Vertex numbering.  Before the snap fix-up, vertex slots are the crossed grid
// edges in point-word order; within a word, x edges, then y edges, then z
// edges, each by ascending z.  A per-word entry holds the word's vertex offset
// within its block of words and popc of its x and y edge masks, so any edge's
// slot is its block offset + entry + popc of the lower bits of its mask.
// Faces come in the reference's order: cells ascending, table slots in order.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

struct McParams {
    const float* vals;
    int nx, ny, nz;
    float amin[3], asize[3];  // asize = aabb_max - aabb_min, rounded in FP32
    float level;
    int method;  // 0 nagae, 1 lorensen
    // outputs
    float* vout;     // [capV, 3]
    int32_t* fout;   // [capF, 3]
    long long capV, capF;
    long long* counts;  // device [0] V, [1] F
    int* status;        // device status word
    long long* vedge;   // optional [capV]: per vertex, 3 * (low endpoint's point id) + axis
};

// Threads per CTA of the emit kernel (128 or 256).
int mc_set_block(int threads);
int mc_get_block();

size_t mc_workspace_bytes(int nx, int ny, int nz, long long capV, long long capF);
int mc_launch(const McParams& p, void* workspace, size_t ws_bytes, cudaStream_t stream);

// Sign bitmap of a grid (also used by dual contouring).
// zero / nzero: 8-byte words to clear before the pass's end (the MC call's
// counters), or nullptr / 0.
void mc_signs_launch(const float* vals, int nx, int ny, int nz, float level, uint32_t* out,
                     cudaStream_t st, unsigned long long* zero = nullptr, long long nzero = 0);

// Bound on an edge parameter t within which a vertex can land on an endpoint's
// position (and so meet another edge's vertex): tau = 2^-20 (1 + max|coord| / h),
// 1 when the grid is too fine for FP32.  asize = aabb_max - aabb_min.
float snap_tau_box(int nx, int ny, int nz, const float* amin, const float* asize);
