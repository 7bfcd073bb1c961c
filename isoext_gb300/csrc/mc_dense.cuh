// Dense-grid marching cubes: tile geometry, workspace layout and launch API.
//
// Tiling.  Grid points (nx, ny, nz; z fastest) are split into tiles
// (plane P, row group rt, z chunk zt).  A tile owns
//   * the points of plane P, rows [rt*R, rt*R + R), z [zt*ZC, zt*ZC + ZC),
//   * every vertex whose key point is one of those points, where a vertex key is
//     (high endpoint of its grid edge, axis), or (grid point, corner) for an
//     edge vertex that rounds exactly onto a grid point,
//   * every cell whose highest corner (v7) is one of those points.
// With R == 1 whenever the z range is split, both the tile's points and its
// cells are contiguous runs of the global point / cell order, so tile order is
// the output order: faces come out in ascending cell id (the reference's
// order, src/mc/mc.cu:33-56) and vertices in ascending key order.
#pragma once

#include <cstdint>

struct McTiles {
    int nx, ny, nz;
    int R;     // point rows per tile
    int ZC;    // z points per tile (multiple of 32); == roundup32(nz) when nZT == 1
    int nRT;   // row groups
    int nZT;   // z chunks
    int RY;    // slab rows = R + 2
    int NW;    // bitmap words per slab row = ZC / 32 + 2
    int CZP;   // value floats per slab row = ZC + 12
    int S;     // slab ring depth (>= 4)
    int PC;    // planes per work item
    int nChunks;
    long long nTiles;  // nx * nRT * nZT
    long long nItems;  // nChunks * nRT * nZT
    int threads;       // threads per CTA
    int ctasPerSm;
    size_t smemBytes;
};

// Per-tile record written by the extract kernel.
struct McTileRec {
    uint32_t vOff, vCnt;  // vertices in the staging buffer
    uint32_t fOff, fCnt;  // faces in the staging buffer
};

struct McParams {
    const float* vals;
    float amin[3], asize[3];
    float level;
    int method;  // 0 nagae, 1 lorensen
    // An edge vertex can round exactly onto a grid point only when its
    // parameter t is within snapTau of 0 or 1 (set by mc_snap_tau); such
    // edges get the exact test.
    float snapTau;
    McTiles t;
    // workspace
    McTileRec* rec;                 // nTiles
    uint2* pre;                     // nTiles: exclusive (V, F) prefix
    float4* sv;                     // staged vertices: x, y, z, key bits
    uint32_t* sf;                   // staged faces: 3 key references each
    unsigned long long* ctr;        // [0] items ticket, [1] V alloc, [2] F alloc
    unsigned long long* blk;        // per 1024 tiles: (sum V, sum F)
    uint32_t* signs;                // sign bitmap [nx][ny][ceil(nz / 32)]
    long long nBlk;                 // number of 1024-tile blocks
    unsigned long long blkV, blkF;  // staging block sizes handed to a CTA at a time
    int* status;                    // device status word
    long long capSV, capSF;         // staging capacities
    // outputs
    float* vout;                    // [capV, 3]
    int32_t* fout;                  // [capF, 3]
    long long capV, capF;
    long long* counts;              // [0] V, [1] F (device)
};

// Host side: choose the tiling for a grid (R, ZC, S and threads come from the
// autotuner or its defaults).
int mc_plan_tiles(int nx, int ny, int nz, int rows, int slabs, int threads, int zchunk,
                  int sm_count, McTiles* out);
size_t mc_workspace_bytes(const McTiles& t, long long capV, long long capF);
float mc_snap_tau(const float amin[3], const float amax[3], const int n[3]);
int mc_launch(const McParams& p, void* workspace, size_t ws_bytes, cudaStream_t stream);
