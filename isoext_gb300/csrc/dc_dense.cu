// Dual contouring on a dense grid (sm_103a).
//
// Steps (each a C entry point; the Python layer sizes buffers between them):
//   classify   sign bitmap (mc_signs) and, per 32-cell word, the number of
//              active cells and crossings, summed per block of 1024 words.
//   intersect  crossing points (lerp, the reference's arithmetic), optional
//              normals from the cell's trilinear interpolant, active cell ids
//              and CSR offsets -- isoext's Intersection (src/its.cu:94-283).
//   solve      per active cell: QEF normal equations accumulated in the
//              reference's order (src/dc.cu:14-65), a register-resident 3x3
//              symmetric Jacobi solve in FP32 with the reference's pseudo-inverse
//              threshold (src/batched_la.cu:152-178) refined once with a
//              double-FP32 residual, clipped to the cell (src/dc.cu:82-99).
//   quads      crossed grid edges in the reference's quad order (by low
//              endpoint, then z, y, x edge; src/grid/uniform.cu:60-83), their 4
//              cells, orientation and diagonal split (src/dc.cu:101-157).
//   weld       dual vertices used by faces, merged by exact position with a
//              hash table (isoext welds by sorted position, src/utils.cu:32-59).
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "dc_common.cuh"
#include "profile.cuh"

namespace {

constexpr int DC_BLOCK = 1024;

// Sign words of a grid row (x, y), aligned to z = 0.
__device__ __forceinline__ const uint32_t* srow(const uint32_t* S, const Grid3& g, int x, int y) {
    const int NWg = (g.nz + 31) / 32;
    return S + ((long long)x * g.ny + y) * NWg;
}
__device__ __forceinline__ uint32_t word_or0(const uint32_t* row, int w, int nw) {
    return (w >= 0 && w < nw) ? row[w] : 0u;
}

// Active-cell mask of cell word (cx, cy, w): cells z in [32w, 32w+32).
__device__ __forceinline__ uint32_t cell_act(const uint32_t* S, const Grid3& g, int cx, int cy, int w,
                                             uint32_t* cw8) {
    const int NWg = (g.nz + 31) / 32;
    uint32_t and8 = ~0u, or8 = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t* r = srow(S, g, cx + (k >> 1), cy + (k & 1));
        const uint32_t a = r[w];
        const uint32_t b = __funnelshift_r(a, word_or0(r, w + 1, NWg), 1);  // bit z <- z + 1
        cw8[2 * k] = a;
        cw8[2 * k + 1] = b;
        and8 &= a & b;
        or8 |= a | b;
    }
    return (or8 & ~and8) & iso::range_mask(w, 0, g.nz - 2);  // cells z <= nz - 2
}
// Case bits of cell at bit b of a cell word, from the 8 corner words cw8
// (index 2k = dz 0, 2k+1 = dz 1 for (dx, dy) = (k >> 1, k & 1)).
__device__ __forceinline__ uint32_t case_of(const uint32_t* cw8, int b) {
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int dx = k >> 1, dy = k & 1;
        cs |= ((cw8[2 * k] >> b) & 1u) << (4 * dx + 2 * dy);
        cs |= ((cw8[2 * k + 1] >> b) & 1u) << (4 * dx + 2 * dy + 1);
    }
    return cs;
}

// Crossings of the active cells of a cell word: the edge table's crossed
// edges are exactly the edges whose corners differ in sign, and corner j's sign
// word is cw8[j], so this is a sum of 12 popcounts.
__device__ __forceinline__ uint32_t word_crossings(const uint32_t* cw8, uint32_t act) {
    uint32_t nk = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) nk += __popc((cw8[iso_edge_corner(2 * e)] ^ cw8[iso_edge_corner(2 * e + 1)]) & act);
    return nk;
}

// Block-wide exclusive scan of two values per thread (NT threads, a multiple
// of 32).
template <int NT = DC_BLOCK>
__device__ __forceinline__ void block_scan2(uint32_t a, uint32_t b, uint32_t& ea, uint32_t& eb,
                                            uint32_t& ta, uint32_t& tb, uint32_t* sm /*66*/) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t ia = a, ib = b;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t x = __shfl_up_sync(~0u, ia, d), y = __shfl_up_sync(~0u, ib, d);
        if (lane >= d) { ia += x; ib += y; }
    }
    if (lane == 31) { sm[warp] = ia; sm[32 + warp] = ib; }
    __syncthreads();
    if (warp == 0) {
        constexpr int NWARP = NT / 32;
        uint32_t x = lane < NWARP ? sm[lane] : 0u, y = lane < NWARP ? sm[32 + lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, x, d), v = __shfl_up_sync(~0u, y, d);
            if (lane >= d) { x += u; y += v; }
        }
        sm[lane] = x;
        sm[32 + lane] = y;
    }
    __syncthreads();
    ea = (warp ? sm[warp - 1] : 0u) + ia - a;
    eb = (warp ? sm[32 + warp - 1] : 0u) + ib - b;
    ta = sm[31];
    tb = sm[63];
    __syncthreads();
}

// ---------------------------------------------------------------------------
// classify: per cell word, active cells and crossings; block sums.

__global__ void __launch_bounds__(DC_BLOCK) dc_cell_count(const uint32_t* __restrict__ S, Grid3 g,
                                                          long long nwords,
                                                          unsigned long long* __restrict__ blk) {
    __shared__ uint32_t sm[66];
    const long long i = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    uint32_t na = 0, nk = 0;
    if (i < nwords) {
        const int NWc = (g.nz - 1 + 31) / 32;
        const int w = int(i % NWc);
        const long long r = i / NWc;
        const int cy = int(r % (g.ny - 1)), cx = int(r / (g.ny - 1));
        uint32_t cw8[8];
        const uint32_t act = cell_act(S, g, cx, cy, w, cw8);
        na = __popc(act);
        nk = word_crossings(cw8, act);
    }
    uint32_t ea, ek, ta, tk;
    block_scan2(na, nk, ea, ek, ta, tk, sm);
    if (threadIdx.x == 0) {
        blk[2 * blockIdx.x] = ta;
        blk[2 * blockIdx.x + 1] = tk;
    }
}

// Exclusive scan of block sums (one CTA; pairs of u64).
__global__ void __launch_bounds__(1024) dc_block_scan(unsigned long long* blk, long long nblk,
                                                      long long* totals) {
    __shared__ unsigned long long wa[32], wb[32], carry[2];
    iso::grid_wait();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) { carry[0] = 0; carry[1] = 0; }
    __syncthreads();
    for (long long base = 0; base < nblk; base += 1024) {
        const long long i = base + tid;
        const unsigned long long a = i < nblk ? blk[2 * i] : 0ull, b = i < nblk ? blk[2 * i + 1] : 0ull;
        unsigned long long ia = a, ib = b;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long x = __shfl_up_sync(~0u, ia, d), y = __shfl_up_sync(~0u, ib, d);
            if (lane >= d) { ia += x; ib += y; }
        }
        if (lane == 31) { wa[warp] = ia; wb[warp] = ib; }
        __syncthreads();
        if (warp == 0) {
            unsigned long long x = wa[lane], y = wb[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long u = __shfl_up_sync(~0u, x, d), v = __shfl_up_sync(~0u, y, d);
                if (lane >= d) { x += u; y += v; }
            }
            wa[lane] = x;
            wb[lane] = y;
        }
        __syncthreads();
        const unsigned long long ea = carry[0] + (warp ? wa[warp - 1] : 0ull) + ia - a;
        const unsigned long long eb = carry[1] + (warp ? wb[warp - 1] : 0ull) + ib - b;
        if (i < nblk) { blk[2 * i] = ea; blk[2 * i + 1] = eb; }
        __syncthreads();
        if (tid == 0) { carry[0] += wa[31]; carry[1] += wb[31]; }
        __syncthreads();
    }
    if (tid == 0) { totals[0] = (long long)carry[0]; totals[1] = (long long)carry[1]; }
}

// ---------------------------------------------------------------------------
// intersect: crossing points / normals, active cells, CSR offsets; also the
// per-word active mask and exclusive active-cell prefix used by the quads.

__global__ void __launch_bounds__(DC_BLOCK) dc_intersect(const float* __restrict__ vals,
                                                         const uint32_t* __restrict__ S, Grid3 g,
                                                         float level, long long nwords,
                                                         const unsigned long long* __restrict__ blk,
                                                         uint32_t* __restrict__ actm,
                                                         uint32_t* __restrict__ offA, float* points,
                                                         float* normals, uint32_t* cell_ids,
                                                         uint32_t* cell_off, long long A, long long K,
                                                         const long long* __restrict__ dn) {
    __shared__ uint32_t sm[66];
    if (dn) {  // the sizes on the device (A, K); 0 when they exceeded the capacities
        A = dn[0];
        K = dn[1];
    }
    const long long i = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    const int NWc = (g.nz - 1 + 31) / 32;
    uint32_t act = 0, na = 0, nk = 0;
    uint32_t cw8[8];
    int cx = 0, cy = 0, w = 0;
    if (i < nwords) {
        w = int(i % NWc);
        const long long r = i / NWc;
        cy = int(r % (g.ny - 1));
        cx = int(r / (g.ny - 1));
        act = cell_act(S, g, cx, cy, w, cw8);
        na = __popc(act);
        nk = word_crossings(cw8, act);
    }
    uint32_t ea, ek, ta, tk;
    block_scan2(na, nk, ea, ek, ta, tk, sm);
    if (i >= nwords) return;
    const unsigned long long a0 = blk[2 * blockIdx.x] + ea, k0 = blk[2 * blockIdx.x + 1] + ek;
    actm[i] = act;
    offA[i] = uint32_t(a0);
    if (!act || !cell_ids) return;
    // active cells of the word: id and the offset of their crossings (values are
    // read by dc_points, one thread per active cell)
    unsigned long long a = a0, k = k0;
    if (a0 >= (unsigned long long)A) return;
    while (act) {
        const int b = __ffs(act) - 1;
        act &= act - 1;
        const int cz = 32 * w + b;
        cell_ids[a] = uint32_t(((long long)cx * (g.ny - 1) + cy) * (g.nz - 1) + cz);
        cell_off[a] = uint32_t(k);
        k += __popc(uint32_t(ISO_EDGE_STATUS[case_of(cw8, b)]));
        ++a;
    }
    if (a == (unsigned long long)A) cell_off[A] = uint32_t(K);
}

// Crossing points (lerp with the reference's arithmetic) and optional normals of
// each active cell's crossed edges, in edge order (src/its.cu:94-159, 186-268).
__global__ void __launch_bounds__(256) dc_points(const float* __restrict__ vals, Grid3 g, float level,
                                                 const uint32_t* __restrict__ cell_ids,
                                                 const uint32_t* __restrict__ cell_off, long long A,
                                                 float* __restrict__ points, float* __restrict__ normals) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const uint32_t cid = cell_ids[a];
    const int cz = int(cid % uint32_t(g.nz - 1));
    const uint32_t rr = cid / uint32_t(g.nz - 1);
    const int cy = int(rr % uint32_t(g.ny - 1)), cx = int(rr / uint32_t(g.ny - 1));
    CellCorners cc;
    load_cell(vals, g, cx, cy, cz, cc);
    uint32_t cs = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) cs |= uint32_t(iso::below(cc.v[j], level)) << j;
    const uint32_t est = edge_status(cs);
    unsigned long long k = cell_off[a];
#pragma unroll 1
    for (uint32_t em = est; em; em &= em - 1) {  // this lane's crossed edges, ascending
        const int e = __ffs(em) - 1;
        float p[3];
        edge_cross(cc, level, e, p);
        points[3 * k + 0] = p[0];
        points[3 * k + 1] = p[1];
        points[3 * k + 2] = p[2];
        if (normals) {
            float n[3];
            cell_normal(cc, p, n);
            normals[3 * k + 0] = n[0];
            normals[3 * k + 1] = n[1];
            normals[3 * k + 2] = n[2];
        }
        ++k;
    }
}

// Normals of an existing intersection from the grid (isoext computes them
// when dual_contouring is given an intersection without normals).
__global__ void dc_normals(const float* __restrict__ vals, Grid3 g, const float* __restrict__ points,
                           const uint32_t* __restrict__ cell_ids, const uint32_t* __restrict__ cell_off,
                           long long A, float* normals) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const uint32_t cid = cell_ids[a];
    const int cz = int(cid % uint32_t(g.nz - 1));
    const uint32_t r = cid / uint32_t(g.nz - 1);
    const int cy = int(r % uint32_t(g.ny - 1)), cx = int(r / uint32_t(g.ny - 1));
    CellCorners cc;
    load_cell(vals, g, cx, cy, cz, cc);
    for (uint32_t k = cell_off[a]; k < cell_off[a + 1]; ++k) {
        const float p[3] = {points[3 * k], points[3 * k + 1], points[3 * k + 2]};
        float n[3];
        cell_normal(cc, p, n);
        normals[3 * k] = n[0];
        normals[3 * k + 1] = n[1];
        normals[3 * k + 2] = n[2];
    }
}

// Whether faces use the dual vertex of active cell (cx, cy, cz) with crossed
// edges est: some crossed edge has all four of its cells inside the grid (then
// its quad is emitted).  Cells at least one cell away from the grid's faces
// have only such edges.
__device__ __forceinline__ bool cell_used(const Grid3& g, int cx, int cy, int cz, uint32_t est) {
    if (cx >= 1 && cx <= g.nx - 3 && cy >= 1 && cy <= g.ny - 3 && cz >= 1 && cz <= g.nz - 3) return est != 0;
    for (uint32_t em = est; em; em &= em - 1) {
        const int e = __ffs(em) - 1;
        const int ca = edge_ca(e), ax = ca ^ edge_cb(e);  // 4 x, 2 y, 1 z
        const int x = cx + (ca >> 2), y = cy + ((ca >> 1) & 1), z = cz + (ca & 1);
        const bool okx = ax == 4 || (x >= 1 && x <= g.nx - 2);
        const bool oky = ax == 2 || (y >= 1 && y <= g.ny - 2);
        const bool okz = ax == 1 || (z >= 1 && z <= g.nz - 2);
        if (okx && oky && okz) return true;
    }
    return false;
}

// Crossings, grid normals and the QEF solve of each active cell in one pass,
// when nobody asked for the intersection: the same arithmetic as dc_points
// followed by dc_solve, without writing points and normals.  used (optional):
// per cell, 0 when no face uses its dual vertex, else 1, or 3 when the vertex
// lies on a face of the cell's box.  F: the arithmetic reading (g.fma), a
// template argument so that each reading compiles without the other's code.
// gc (optional): the grid's coordinates (x, y, z).
template <bool F>
__global__ void __launch_bounds__(256) dc_cell_solve(const float* __restrict__ vals, Grid3 g, float level,
                                                     const uint32_t* __restrict__ cell_ids, long long A, float reg,
                                                     float svd_tol, float* __restrict__ dual,
                                                     const long long* __restrict__ dn,
                                                     uint8_t* __restrict__ used, const float* __restrict__ gc) {
    iso::grid_wait();
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (dn) A = dn[0];
    if (a >= A) return;
    const uint32_t cid = cell_ids[a];
    const int cz = int(cid % uint32_t(g.nz - 1));
    const uint32_t rr = cid / uint32_t(g.nz - 1);
    const int cy = int(rr % uint32_t(g.ny - 1)), cx = int(rr / uint32_t(g.ny - 1));
    g.fma = F;
    CellCorners cc;
    if (gc) load_cell_table(vals, g, gc, cx, cy, cz, cc);
    else load_cell(vals, g, cx, cy, cz, cc);
    uint32_t cs = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) cs |= uint32_t(iso::below(cc.v[j], level)) << j;
    const uint32_t est = edge_status(cs);
    const bool is_used = used && cell_used(g, cx, cy, cz, est);
    Qef Q;
    qef_init(Q, g.fma);
    uint32_t K = 0;
#pragma unroll 1
    for (uint32_t em = est; em; em &= em - 1) {  // this lane's crossed edges, ascending
        const int e = __ffs(em) - 1;
        float p[3], n[3];
        edge_cross(cc, level, e, p);
        cell_normal(cc, p, n);
        qef_add(Q, p[0], p[1], p[2], n[0], n[1], n[2]);
        ++K;
    }
    qef_finish(Q, K, reg, svd_tol);
    bool face = false;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float lo = cc.p[0][q], hi = cc.p[7][q];  // the cell's box
        const float x = fminf(fmaxf(float(Q.x[q]), lo), hi);
        face |= x == lo || x == hi;
        dual[3 * a + q] = x;
    }
    if (used) used[a] = is_used ? (face ? 3 : 1) : 0;  // bit 1: on a face of its cell's box
}

// The solve for the call's arithmetic reading.
using SolveFn = void (*)(const float*, Grid3, float, const uint32_t*, long long, float, float, float*,
                         const long long*, uint8_t*, const float*);
SolveFn solve_kernel(const Grid3& g) { return g.fma ? dc_cell_solve<true> : dc_cell_solve<false>; }

// Lane whose inclusive prefix first exceeds j (prefixes nondecreasing, j < total).
__device__ __forceinline__ int owner_lane(uint32_t incl, uint32_t j) {
    int lo = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const uint32_t pv = __shfl_sync(~0u, incl, lo + s - 1);
        if (pv <= j) lo += s;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// solve

__global__ void dc_solve(const float* __restrict__ points, const float* __restrict__ normals,
                         const uint32_t* __restrict__ cell_ids, const uint32_t* __restrict__ cell_off,
                         long long A, Grid3 g, float reg, float svd_tol, float* dual) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const uint32_t k0 = cell_off[a], k1 = cell_off[a + 1];
    Qef Q;
    qef_solve(points + 3ll * k0, normals + 3ll * k0, k1 - k0, reg, svd_tol, g.fma, Q);
    const double* x = Q.x;
    // clip to the cell box (corner 0 .. corner 7)
    const uint32_t cid = cell_ids[a];
    const uint32_t cz = cid % uint32_t(g.nz - 1);
    const uint32_t rr = cid / uint32_t(g.nz - 1);
    const uint32_t cy = rr % uint32_t(g.ny - 1), cx = rr / uint32_t(g.ny - 1);
    const uint32_t ci[3] = {cx, cy, cz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float lo = coord(g, k, ci[k]), hi = coord(g, k, ci[k] + 1);
        dual[3 * a + k] = fminf(fmaxf(float(x[k]), lo), hi);
    }
}

// ---------------------------------------------------------------------------
// quads

// Crossed edges with a complete quad, per point word (points z in [32w, 32w+32)
// of row (x, y)), as masks for the z, y and x edges leaving each point.
__device__ __forceinline__ void quad_masks(const uint32_t* S, const Grid3& g, int x, int y, int w,
                                           uint32_t& mz, uint32_t& my, uint32_t& mx) {
    const int NWg = (g.nz + 31) / 32;
    const uint32_t* r = srow(S, g, x, y);
    const uint32_t s = r[w];
    // z edge (z -> z+1): cells (x-1..x, y-1..y, z)
    mz = my = mx = 0;
    const uint32_t zin = iso::range_mask(w, 1, g.nz - 2);     // 1 <= z <= nz-2
    const uint32_t zall = iso::range_mask(w, 0, g.nz - 2);    // z <= nz-2 (edge exists)
    if (x >= 1 && x <= g.nx - 2 && y >= 1 && y <= g.ny - 2)
        mz = (s ^ __funnelshift_r(s, word_or0(r, w + 1, NWg), 1)) & zall;
    // y edge (y -> y+1): cells (x-1..x, y, z-1..z)
    if (x >= 1 && x <= g.nx - 2 && y <= g.ny - 2) my = (s ^ srow(S, g, x, y + 1)[w]) & zin;
    // x edge (x -> x+1): cells (x, y-1..y, z-1..z)
    if (x <= g.nx - 2 && y >= 1 && y <= g.ny - 2) mx = (s ^ srow(S, g, x + 1, y)[w]) & zin;
}

__global__ void __launch_bounds__(DC_BLOCK) dc_quad_count(const uint32_t* __restrict__ S, Grid3 g,
                                                          long long nwords,
                                                          unsigned long long* __restrict__ blk) {
    __shared__ uint32_t sm[66];
    const long long i = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    uint32_t nq = 0;
    if (i < nwords) {
        const int NWg = (g.nz + 31) / 32;
        const int w = int(i % NWg);
        const long long r = i / NWg;
        const int y = int(r % g.ny), x = int(r / g.ny);
        uint32_t mz, my, mx;
        quad_masks(S, g, x, y, w, mz, my, mx);
        nq = __popc(mz) + __popc(my) + __popc(mx);
    }
    uint32_t e0, e1, t0, t1;
    block_scan2(nq, 0u, e0, e1, t0, t1, sm);
    if (threadIdx.x == 0) {
        blk[2 * blockIdx.x] = t0;
        blk[2 * blockIdx.x + 1] = 0;
    }
}

// Active index of cell (cx, cy, cz): prefix of its word + active cells below it.
__device__ __forceinline__ uint32_t active_index(const uint32_t* actm, const uint32_t* offA,
                                                 const Grid3& g, int cx, int cy, int cz) {
    const int NWc = (g.nz - 1 + 31) / 32;
    const long long wi = ((long long)cx * (g.ny - 1) + cy) * NWc + (cz >> 5);
    return offA[wi] + __popc(actm[wi] & ((1u << (cz & 31)) - 1u));
}

// |a - b| (norm(v0 - v2) of src/dc.cu:139), in the grid's arithmetic reading.
__device__ __forceinline__ float dist3(const float* a, const float* b, bool fma) {
    const float dx = __fsub_rn(a[0], b[0]), dy = __fsub_rn(a[1], b[1]), dz = __fsub_rn(a[2], b[2]);
    return iso::norm3f(dx, dy, dz, fma);
}

// The k-th quad of a point word in the reference's order: by bit (low endpoint
// z) ascending, then the bit's z, y, x edges.
__device__ __forceinline__ void kth_quad(uint32_t mz, uint32_t my, uint32_t mx, uint32_t k, int& b, int& ax) {
    int lo = 0;  // largest lo with (quads of bits < lo) <= k
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const uint32_t m = (1u << (lo + s)) - 1u;  // lo + s <= 31
        if (uint32_t(__popc(mz & m) + __popc(my & m) + __popc(mx & m)) <= k) lo += s;
    }
    b = lo;
    const uint32_t below = (1u << lo) - 1u;
    uint32_t r = k - uint32_t(__popc(mz & below) + __popc(my & below) + __popc(mx & below));
    ax = 0;
    if ((mz >> b) & 1u) {
        if (r == 0) { ax = 2; return; }
        --r;
    }
    if ((my >> b) & 1u) {
        if (r == 0) { ax = 1; return; }
    }
}

// The quads of a block of point words, handed out over the lanes of each warp
// (a word has 0 .. 96 of them): every lane emits one quad per round.
__global__ void __launch_bounds__(DC_BLOCK) dc_quad_emit(const uint32_t* __restrict__ S, Grid3 g,
                                                         long long nwords,
                                                         const unsigned long long* __restrict__ blk,
                                                         const uint32_t* __restrict__ actm,
                                                         const uint32_t* __restrict__ offA,
                                                         const float* __restrict__ dual,
                                                         int32_t* __restrict__ tri,
                                                         const long long* __restrict__ dn) {
    __shared__ uint32_t sm[66];
    const long long i = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    const int NWg = (g.nz + 31) / 32;
    const int lane = threadIdx.x & 31;
    // dn: the triangle indices the output holds (6 Q, or 0 over capacity)
    const unsigned long long qmax = dn ? (unsigned long long)(dn[2] / 6) : ~0ull;
    uint32_t mz = 0, my = 0, mx = 0, sw = 0;
    int x = 0, y = 0, w = 0;
    if (i < nwords) {
        w = int(i % NWg);
        const long long r = i / NWg;
        y = int(r % g.ny);
        x = int(r / g.ny);
        quad_masks(S, g, x, y, w, mz, my, mx);
        sw = srow(S, g, x, y)[w];
    }
    const uint32_t nq = __popc(mz) + __popc(my) + __popc(mx);
    uint32_t eq, e1, tq, t1;
    block_scan2(nq, 0u, eq, e1, tq, t1, sm);
    const unsigned long long qb = blk[2 * blockIdx.x];
    uint32_t incl = nq;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(~0u, incl, d);
        if (lane >= d) incl += t;
    }
    const uint32_t total = __shfl_sync(~0u, incl, 31);
    for (uint32_t rr = 0; rr < total; rr += 32) {
        const uint32_t j = rr + lane;
        const int o = owner_lane(incl, min(j, total - 1));
        const uint32_t oexcl = __shfl_sync(~0u, incl - nq, o), oeq = __shfl_sync(~0u, eq, o);
        const uint32_t omz = __shfl_sync(~0u, mz, o), omy = __shfl_sync(~0u, my, o), omx = __shfl_sync(~0u, mx, o);
        const uint32_t os = __shfl_sync(~0u, sw, o);
        const int ox = __shfl_sync(~0u, x, o), oy = __shfl_sync(~0u, y, o), ow = __shfl_sync(~0u, w, o);
        if (j >= total) continue;
        const uint32_t k = j - oexcl;
        const unsigned long long q = qb + oeq + k;
        if (q >= qmax) continue;
        int b, ax;
        kth_quad(omz, omy, omx, k, b, ax);
        const int z = 32 * ow + b;
        // is_out = v(p0) <= v(p1): for a crossed edge this holds exactly when
        // the low endpoint p0 is below the level
        const bool out = (os >> b) & 1u;
        // edge_neighbors_table (src/shared_luts.cu:78-81): the 4 cells are p - o_i
        int c[4][3];
        if (ax == 0) {
            const int off[4][3] = {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}};
            for (int t = 0; t < 4; ++t) { c[t][0] = ox - off[t][0]; c[t][1] = oy - off[t][1]; c[t][2] = z - off[t][2]; }
        } else if (ax == 1) {
            const int off[4][3] = {{0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 0, 0}};
            for (int t = 0; t < 4; ++t) { c[t][0] = ox - off[t][0]; c[t][1] = oy - off[t][1]; c[t][2] = z - off[t][2]; }
        } else {
            const int off[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
            for (int t = 0; t < 4; ++t) { c[t][0] = ox - off[t][0]; c[t][1] = oy - off[t][1]; c[t][2] = z - off[t][2]; }
        }
        int32_t qi[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) qi[t] = int32_t(active_index(actm, offA, g, c[t][0], c[t][1], c[t][2]));
        if (!out) {
            const int32_t t0 = qi[0], t1q = qi[1];
            qi[0] = qi[3]; qi[1] = qi[2]; qi[2] = t1q; qi[3] = t0;
        }
        float v[4][3];
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int a = 0; a < 3; ++a) v[t][a] = dual[3 * (long long)qi[t] + a];
        int32_t* o6 = tri + 6 * q;
        if (dist3(v[0], v[2], g.fma) > dist3(v[1], v[3], g.fma)) {
            o6[0] = qi[1]; o6[1] = qi[3]; o6[2] = qi[0];
            o6[3] = qi[3]; o6[4] = qi[1]; o6[5] = qi[2];
        } else {
            o6[0] = qi[2]; o6[1] = qi[0]; o6[2] = qi[1];
            o6[3] = qi[0]; o6[4] = qi[2]; o6[5] = qi[3];
        }
    }
}

// ---------------------------------------------------------------------------
// weld: exact-position dedup of the dual vertices faces use.

using iso::pos_bits;
using iso::pos_hash;

__global__ void dc_mark_used(const int32_t* __restrict__ tri, long long n, uint32_t* used,
                             const long long* __restrict__ dn) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (dn) n = dn[2];
    if (i < n) used[tri ? tri[i] : int32_t(i)] = 1u;  // tri == nullptr: triangle i is point i
}

// Probes before an insert gives up (the table is at most half full when the
// caller's capacity holds the distinct positions; past it the status says
// overflow and the counts give a size that fits).  Once the status says
// overflow, later threads skip their probes: the call's output is discarded.
constexpr uint32_t HASH_PROBES = 512;

// Insert used vertices (used == nullptr: all); a slot keeps the smallest index
// with its position.
__global__ void dc_hash_insert(const float* __restrict__ dual, const uint32_t* __restrict__ used,
                               long long A, uint32_t* table, uint32_t mask, int* status,
                               const long long* __restrict__ dn) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (dn) A = dn[0];
    if (a >= A || (used && !used[a])) return;
    if (status && *(volatile int*)status == int(ISO_ERR_OVERFLOW)) return;
    const uint32_t k0 = pos_bits(dual[3 * a]), k1 = pos_bits(dual[3 * a + 1]), k2 = pos_bits(dual[3 * a + 2]);
    uint32_t h = pos_hash(k0, k1, k2) & mask;
    for (uint32_t probe = 0; probe <= mask && probe < HASH_PROBES; ++probe, h = (h + 1) & mask) {
        const uint32_t cur = atomicCAS(&table[h], 0xffffffffu, uint32_t(a));
        if (cur == 0xffffffffu) return;
        const uint32_t j = cur;
        if (pos_bits(dual[3ll * j]) == k0 && pos_bits(dual[3ll * j + 1]) == k1 &&
            pos_bits(dual[3ll * j + 2]) == k2) {
            atomicMin(&table[h], uint32_t(a));
            return;
        }
    }
    if (status) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
}

// rep[a] = smallest index with the same position (for used vertices).
__global__ void dc_hash_lookup(const float* __restrict__ dual, const uint32_t* __restrict__ used,
                               long long A, const uint32_t* __restrict__ table, uint32_t mask,
                               uint32_t* rep, const long long* __restrict__ dn) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (dn) A = dn[0];
    if (a >= A) return;
    if (used && !used[a]) { rep[a] = 0xffffffffu; return; }
    const uint32_t k0 = pos_bits(dual[3 * a]), k1 = pos_bits(dual[3 * a + 1]), k2 = pos_bits(dual[3 * a + 2]);
    uint32_t h = pos_hash(k0, k1, k2) & mask;
    for (uint32_t probe = 0; probe <= mask && probe < HASH_PROBES; ++probe, h = (h + 1) & mask) {
        const uint32_t j = table[h];
        if (j == 0xffffffffu) break;
        if (pos_bits(dual[3ll * j]) == k0 && pos_bits(dual[3ll * j + 1]) == k1 &&
            pos_bits(dual[3ll * j + 2]) == k2) {
            rep[a] = j;
            return;
        }
    }
    rep[a] = uint32_t(a);
}

// Per block of 1024 dual vertices: number of representatives (rep[a] == a).
__global__ void __launch_bounds__(DC_BLOCK) dc_rep_count(const uint32_t* __restrict__ rep, long long A,
                                                         unsigned long long* blk, const long long* __restrict__ dn) {
    __shared__ uint32_t sm[66];
    const long long a = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    if (dn) A = dn[0];
    const uint32_t is = (a < A && rep[a] == uint32_t(a)) ? 1u : 0u;
    uint32_t e0, e1, t0, t1;
    block_scan2(is, 0u, e0, e1, t0, t1, sm);
    if (threadIdx.x == 0) { blk[2 * blockIdx.x] = t0; blk[2 * blockIdx.x + 1] = 0; }
}

__global__ void __launch_bounds__(DC_BLOCK) dc_rep_write(const uint32_t* __restrict__ rep, long long A,
                                                         const unsigned long long* __restrict__ blk,
                                                         const float* __restrict__ dual, uint32_t* newidx,
                                                         float* vout, uint32_t* vsrc, const long long* __restrict__ dn) {
    __shared__ uint32_t sm[66];
    const long long a = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    if (dn) A = dn[0];
    const uint32_t is = (a < A && rep[a] == uint32_t(a)) ? 1u : 0u;
    uint32_t e0, e1, t0, t1;
    block_scan2(is, 0u, e0, e1, t0, t1, sm);
    if (!is) return;
    const unsigned long long o = blk[2 * blockIdx.x] + e0;
    newidx[a] = uint32_t(o);
    if (dn && (long long)o >= dn[3]) return;  // past the vertex capacity: the caller sees V and retries
    if (vsrc) vsrc[o] = uint32_t(a);
    vout[3 * o] = dual[3 * a];
    vout[3 * o + 1] = dual[3 * a + 1];
    vout[3 * o + 2] = dual[3 * a + 2];
}

__global__ void dc_remap(const int32_t* __restrict__ tri, long long n, const uint32_t* __restrict__ rep,
                         const uint32_t* __restrict__ newidx, int32_t* fout, const long long* __restrict__ dn) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (dn) n = dn[2];
    if (i < n) fout[i] = int32_t(newidx[rep[tri ? tri[i] : int32_t(i)]]);
}


// ---------------------------------------------------------------------------
// One-call dual contouring: after the sign pass, eight kernels chained by
// programmatic dependent launch, with the sizes kept on the device.
//
//   dc_cells_count / _scan / _write
//                  per point word: active cells, crossings, and the quads each
//                  active cell owns.  A quad's owner is the cell whose lowest
//                  corner is the low endpoint of the quad's edge, so the
//                  reference's quad order (low endpoint, then z, y, x edge) is
//                  the owners' order.  Counts per warp, one CTA scans them and
//                  checks the sizes, then the words are written with offsets.
//   dc_cell_solve  the QEF solve and whether faces use the cell.
//   dc_weld_flags / dc_block_scan / dc_weld_number
//                  the exact-position weld.  A dual vertex is clipped to its
//                  cell's closed box, and the boxes of different cells meet only
//                  on shared faces, so a vertex strictly inside its box has a
//                  position of its own, and one on a face can only equal the
//                  vertices of the cells around that face, edge or corner.
//                  Representatives (smallest index of a position) are numbered
//                  in cell order.
//   dc_cell_quads  each active cell's quads with the final vertex numbers.

// Crossed edges of one cell (bit b of a cell word): the 12 corner-sign XORs.
__device__ __forceinline__ uint32_t cell_crossings(const uint32_t* ex, int b) {
    uint32_t n = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) n += (ex[e] >> b) & 1u;
    return n;
}

constexpr int CELLS_THREADS = 256;  // dc_cells: threads per CTA
constexpr int CELLS_WPT = 4;        // point words per thread and round (one 16-byte load per row)
constexpr int CELLS_ROUNDS = 2;
constexpr int CELLS_TILE = CELLS_THREADS * CELLS_WPT * CELLS_ROUNDS;  // point words per CTA

// Owned quad edges of a cell word's active cells: corner 0 to corner 1 (z),
// 2 (y), 4 (x); complete when the edge's other two coordinates are >= 1 (the
// upper bounds hold for every cell).
__device__ __forceinline__ void owned_quads(const Grid3& g, const uint32_t* cw8, uint32_t act, int cx, int cy, int w,
                                            uint32_t& qz, uint32_t& qy, uint32_t& qx) {
    const uint32_t zin = iso::range_mask(w, 1, g.nz - 2);
    qz = (cx >= 1 && cy >= 1) ? (cw8[0] ^ cw8[1]) & act : 0u;
    qy = cx >= 1 ? (cw8[0] ^ cw8[2]) & act & zin : 0u;
    qx = cy >= 1 ? (cw8[0] ^ cw8[4]) & act & zin : 0u;
}

// The sign words pw .. pw+3 of the rows (x, y), (x, y+1), (x+1, y), (x+1, y+1)
// of point word pw (flat offsets 0, syw, sxw, sxw + syw), and each row's word
// pw+4 (the next lane's first word, or a load).  All lanes call it.
struct QuadRows {
    uint32_t r[4][CELLS_WPT];  // row k = 2 dx + dy
    uint32_t n4[4];
};

__device__ __forceinline__ void load_quad_rows(const uint32_t* __restrict__ S, uint32_t pw, uint32_t sxw,
                                               uint32_t syw, uint32_t PW, bool vec, int lane, QuadRows& q) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t o = pw + (k >> 1) * sxw + (k & 1) * syw;
        if (vec && o + CELLS_WPT <= PW) {
            const uint4 v4 = __ldg(reinterpret_cast<const uint4*>(S + o));
            q.r[k][0] = v4.x; q.r[k][1] = v4.y; q.r[k][2] = v4.z; q.r[k][3] = v4.w;
        } else {
#pragma unroll
            for (int j = 0; j < CELLS_WPT; ++j) q.r[k][j] = o + j < PW ? __ldg(S + o + j) : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        q.n4[k] = __shfl_down_sync(~0u, q.r[k][0], 1);
        if (lane == 31) {
            const uint32_t o = pw + CELLS_WPT + (k >> 1) * sxw + (k & 1) * syw;
            q.n4[k] = o < PW ? __ldg(S + o) : 0u;
        }
    }
}

// No cell of the lane's words can be active: all 20 words equal, all 0 or ~0.
__device__ __forceinline__ bool quad_rows_quiet(const QuadRows& q) {
    const uint32_t u = q.r[0][0];
    uint32_t d = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        d |= q.n4[k] ^ u;
#pragma unroll
        for (int j = 0; j < CELLS_WPT; ++j) d |= q.r[k][j] ^ u;
    }
    return (u == 0u || u == ~0u) && d == 0u;
}

// Corner words (cw8[2k]: dz 0, cw8[2k+1]: dz 1) and active cells of word j of
// the lane, point word (x, y, w).
__device__ __forceinline__ uint32_t quad_word_act(const Grid3& g, int nwg, int nwc, const QuadRows& q, int j, int x,
                                                  int y, int w, uint32_t* cw8) {
    const bool nxt = w + 1 < nwg;
    uint32_t and8 = ~0u, or8 = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t a = q.r[k][j];
        const uint32_t nb = nxt ? (j + 1 < CELLS_WPT ? q.r[k][(j + 1) % CELLS_WPT] : q.n4[k]) : 0u;
        const uint32_t b = __funnelshift_r(a, nb, 1);  // bit z <- z + 1
        cw8[2 * k] = a;
        cw8[2 * k + 1] = b;
        and8 &= a & b;
        or8 |= a | b;
    }
    if (x >= g.nx - 1 || y >= g.ny - 1 || w >= nwc) return 0u;
    return (or8 & ~and8) & iso::range_mask(w, 0, g.nz - 2);
}

// Next point word in (x, y, w) order.
__device__ __forceinline__ void next_point_word(const Grid3& g, int nwg, int& x, int& y, int& w) {
    if (++w == nwg) {
        w = 0;
        if (++y == g.ny) { y = 0; ++x; }
    }
}

// Geometry of the flat point-word bitmap, shared by the dc_cells kernels.
struct PwGrid {
    int NWg, NWc;
    uint32_t syw, sxw, PW;  // row stride, plane stride, point words (< 2^32)
    bool vec;               // rows start on 16-byte boundaries
};

__device__ __forceinline__ PwGrid pw_grid(const Grid3& g) {
    PwGrid p;
    p.NWg = (g.nz + 31) / 32;
    p.NWc = (g.nz - 1 + 31) / 32;
    p.syw = uint32_t(p.NWg);
    p.sxw = uint32_t(g.ny) * p.syw;
    p.PW = uint32_t(g.nx) * p.sxw;
    p.vec = (p.NWg & 3) == 0;
    return p;
}

// Round j of a lane of warp gw (over the grid): point words pw .. pw + 3.  A
// warp's rounds are consecutive, so its words are too.
__device__ __forceinline__ uint32_t cells_pw(uint32_t gw, int lane, int j) {
    return gw * uint32_t(32 * CELLS_WPT * CELLS_ROUNDS) + uint32_t(j * 32 * CELLS_WPT) + uint32_t(lane * CELLS_WPT);
}

__device__ __forceinline__ void pw_xyw(const Grid3& g, const PwGrid& p, uint32_t pw, int& x, int& y, int& w) {
    const uint32_t row = pw / p.syw;
    w = int(pw - row * p.syw);
    x = int(row / uint32_t(g.ny));
    y = int(row - uint32_t(x) * uint32_t(g.ny));
}

// Per warp of 256 point words (flat bitmap order (x, y, w), which orders cells
// as their ids do): the active masks (written here), and the counts of active
// cells, owned quads and crossings.  A lane takes 4 consecutive words per
// round: one 16-byte load per row, and a warp whose 128 words are all inside
// or outside skips the rest.  wsum[warp] = the warp's exclusive prefix within
// its CTA and its busy rounds; csum[CTA] = the CTA's sums.
constexpr int CELLS_WARPS = CELLS_THREADS / 32;

__device__ __forceinline__ void store_masks(uint32_t* __restrict__ m, uint32_t pw, uint32_t PW, const uint32_t* v) {
    if (pw + CELLS_WPT <= PW) {
        *reinterpret_cast<uint4*>(m + pw) = make_uint4(v[0], v[1], v[2], v[3]);
    } else {
        for (int k = 0; k < CELLS_WPT; ++k)
            if (pw + k < PW) m[pw + k] = v[k];
    }
}

__global__ void __launch_bounds__(CELLS_THREADS, 4) dc_cells_count(const uint32_t* __restrict__ S, Grid3 g,
                                                                   uint32_t* __restrict__ actm,
                                                                   uint32_t* __restrict__ wsum,
                                                                   uint32_t* __restrict__ csum,
                                                                   float* __restrict__ gc) {
    __shared__ uint32_t ws[3][CELLS_WARPS];
    iso::grid_wait();
    // the grid's coordinates (x, then y, then z), read by the solve
    for (uint32_t i = blockIdx.x * CELLS_THREADS + threadIdx.x; i < uint32_t(g.nx + g.ny + g.nz);
         i += gridDim.x * CELLS_THREADS) {
        const int axis = i < uint32_t(g.nx) ? 0 : (i < uint32_t(g.nx + g.ny) ? 1 : 2);
        const uint32_t k = i - (axis > 0 ? uint32_t(g.nx) : 0u) - (axis > 1 ? uint32_t(g.ny) : 0u);
        gc[i] = coord(g, axis, k);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * CELLS_WARPS + warp;
    const PwGrid p = pw_grid(g);
    uint32_t sa = 0, sq = 0, sk = 0, busy = 0;
    for (int j = 0; j < CELLS_ROUNDS; ++j) {
        const uint32_t pw = cells_pw(gw, lane, j);
        QuadRows q;
        load_quad_rows(S, pw, p.sxw, p.syw, p.PW, p.vec, lane, q);
        uint32_t act[CELLS_WPT] = {0u, 0u, 0u, 0u};
        if (!__all_sync(~0u, quad_rows_quiet(q) || pw >= p.PW)) {
            busy |= 1u << j;
            int x = 0, y = 0, w = 0;
            if (pw < p.PW) pw_xyw(g, p, pw, x, y, w);
#pragma unroll
            for (int k = 0; k < CELLS_WPT; ++k) {
                uint32_t cw8[8];
                act[k] = pw + k < p.PW ? quad_word_act(g, p.NWg, p.NWc, q, k, x, y, w, cw8) : 0u;
                if (act[k]) {
                    uint32_t qz, qy, qx;
                    owned_quads(g, cw8, act[k], x, y, w, qz, qy, qx);
                    sa += __popc(act[k]);
                    sq += __popc(qz) + __popc(qy) + __popc(qx);
                    sk += word_crossings(cw8, act[k]);
                }
                next_point_word(g, p.NWg, x, y, w);
            }
        }
        if (pw < p.PW) store_masks(actm, pw, p.PW, act);
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        sa += __shfl_xor_sync(~0u, sa, d);
        sq += __shfl_xor_sync(~0u, sq, d);
        sk += __shfl_xor_sync(~0u, sk, d);
    }
    if (lane == 0) { ws[0][warp] = sa; ws[1][warp] = sq; ws[2][warp] = sk; }
    __syncthreads();
    if (warp == 0) {
        uint32_t e[3], t[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            const uint32_t x = lane < CELLS_WARPS ? ws[v][lane] : 0u;
            uint32_t incl = x;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t u = __shfl_up_sync(~0u, incl, d);
                if (lane >= d) incl += u;
            }
            e[v] = incl - x;
            t[v] = __shfl_sync(~0u, incl, 31);
        }
        if (lane < CELLS_WARPS) *reinterpret_cast<uint4*>(wsum + 4u * (blockIdx.x * CELLS_WARPS + lane)) =
            make_uint4(e[0], e[1], e[2], 0u);
        if (lane == 0) *reinterpret_cast<uint4*>(csum + 4u * blockIdx.x) = make_uint4(t[0], t[1], t[2], 0u);
    }
    __syncthreads();  // the record's busy word after warp 0's store of the prefixes
    if (lane == 0) wsum[4u * gw + 3] = busy;
}

// One CTA: exclusive scan of the CTAs' (active, quads, crossings) sums in
// place, the totals checked against the capacities.
__global__ void __launch_bounds__(1024) dc_cells_scan(uint32_t* __restrict__ csum, long long ncta, long long capA,
                                                      long long capQ, long long* eff, long long* counts,
                                                      uint32_t* __restrict__ cell_off, int* status) {
    __shared__ unsigned long long part[3][32], carry[3];
    iso::grid_wait();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 3) carry[tid] = 0;
    __syncthreads();
    for (long long base = 0; base < ncta; base += 1024) {
        const long long i = base + tid;
        const uint4 v = i < ncta ? *reinterpret_cast<const uint4*>(csum + 4 * i) : make_uint4(0u, 0u, 0u, 0u);
        const unsigned long long c[3] = {v.x, v.y, v.z};
        unsigned long long in[3] = {v.x, v.y, v.z};
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const unsigned long long u = __shfl_up_sync(~0u, in[t], d);
                if (lane >= d) in[t] += u;
            }
        if (lane == 31)
#pragma unroll
            for (int t = 0; t < 3; ++t) part[t][warp] = in[t];
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                unsigned long long x = part[t][lane];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const unsigned long long u = __shfl_up_sync(~0u, x, d);
                    if (lane >= d) x += u;
                }
                part[t][lane] = x;
            }
        }
        __syncthreads();
        if (i < ncta) {
            unsigned long long e[3];
#pragma unroll
            for (int t = 0; t < 3; ++t) e[t] = carry[t] + (warp ? part[t][warp - 1] : 0ull) + in[t] - c[t];
            // offsets past 2^32 only matter when the sizes overflow (then nothing is used)
            *reinterpret_cast<uint4*>(csum + 4 * i) = make_uint4(uint32_t(e[0]), uint32_t(e[1]), uint32_t(e[2]), 0u);
        }
        __syncthreads();
        if (tid < 3) carry[tid] += part[tid][31];
        __syncthreads();
    }
    if (tid == 0) {
        const long long A = (long long)carry[0], Q = (long long)carry[1], K = (long long)carry[2];
        const bool ok = A <= capA && Q <= capQ && A < 0x7fffffffll && K < 0x7fffffffll && 6 * Q < 0x7fffffffll;
        if (!ok) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
        eff[0] = ok ? A : 0;
        eff[1] = ok ? K : 0;
        eff[2] = ok ? 6 * Q : 0;
        eff[3] = capA;
        counts[0] = 0;
        counts[1] = ok ? 2 * Q : 0;
        counts[2] = A;
        counts[3] = K;
        counts[4] = Q;
        if (cell_off && ok) cell_off[A] = uint32_t(K);
    }
}

// The busy rounds of dc_cells_count again, with each warp's offsets: active
// prefixes per point word (rounds without an active cell have none to look
// up), and per active cell its id, its first owned quad, its owned quad edges
// (bits 0-2: z, y, x) with the sign of its lowest corner (bit 3), and (when
// asked) its first crossing.
__global__ void __launch_bounds__(CELLS_THREADS, 4) dc_cells_write(const uint32_t* __restrict__ S, Grid3 g,
                                                                   const uint32_t* __restrict__ actm,
                                                                   const uint32_t* __restrict__ wsum,
                                                                   const uint32_t* __restrict__ csum,
                                                                   uint32_t* __restrict__ offA,
                                                                   uint32_t* __restrict__ cell_ids,
                                                                   uint32_t* __restrict__ qoff,
                                                                   uint8_t* __restrict__ qbits,
                                                                   uint32_t* __restrict__ cell_off, long long capA) {
    iso::grid_wait();
    const int lane = threadIdx.x & 31;
    const uint32_t gw = blockIdx.x * CELLS_WARPS + (threadIdx.x >> 5);
    const PwGrid p = pw_grid(g);
    const uint4 wo = *reinterpret_cast<const uint4*>(wsum + 4u * gw);
    const uint4 co = *reinterpret_cast<const uint4*>(csum + 4u * blockIdx.x);
    const uint32_t wbusy = wo.w;
    if (!wbusy) return;
    unsigned long long ra = (unsigned long long)co.x + wo.x, rq = (unsigned long long)co.y + wo.y,
                       rk = (unsigned long long)co.z + wo.z;
    const unsigned long long cap = (unsigned long long)capA;  // over capacity the caller reruns
    const bool want_k = cell_off != nullptr;
    for (int j = 0; j < CELLS_ROUNDS; ++j) {
        if (!((wbusy >> j) & 1u)) continue;  // no active cell: nothing to number
        const uint32_t pw = cells_pw(gw, lane, j);
        uint32_t act[CELLS_WPT] = {0u, 0u, 0u, 0u};
        if (pw + CELLS_WPT <= p.PW) {
            const uint4 a4 = *reinterpret_cast<const uint4*>(actm + pw);
            act[0] = a4.x; act[1] = a4.y; act[2] = a4.z; act[3] = a4.w;
        } else {
#pragma unroll
            for (int k = 0; k < CELLS_WPT; ++k) act[k] = pw + k < p.PW ? actm[pw + k] : 0u;
        }
        QuadRows q;
        load_quad_rows(S, pw, p.sxw, p.syw, p.PW, p.vec, lane, q);
        int x = 0, y = 0, w = 0;
        if (pw < p.PW) pw_xyw(g, p, pw, x, y, w);
        const int x0 = x, y0 = y, w0 = w;
        uint32_t la = 0, lq = 0, lk = 0;
#pragma unroll
        for (int k = 0; k < CELLS_WPT; ++k) {
            if (act[k]) {
                uint32_t cw8[8], qz, qy, qx;
                quad_word_act(g, p.NWg, p.NWc, q, k, x, y, w, cw8);
                owned_quads(g, cw8, act[k], x, y, w, qz, qy, qx);
                la += __popc(act[k]);
                lq += __popc(qz) + __popc(qy) + __popc(qx);
                if (want_k) lk += word_crossings(cw8, act[k]);
            }
            next_point_word(g, p.NWg, x, y, w);
        }
        uint32_t ia = la, iq = lq, ik = lk;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t ta = __shfl_up_sync(~0u, ia, d), tq = __shfl_up_sync(~0u, iq, d),
                           tk = __shfl_up_sync(~0u, ik, d);
            if (lane >= d) { ia += ta; iq += tq; ik += tk; }
        }
        unsigned long long a = ra + ia - la, qq = rq + iq - lq, kk = rk + ik - lk;
        ra += __shfl_sync(~0u, ia, 31);
        rq += __shfl_sync(~0u, iq, 31);
        rk += __shfl_sync(~0u, ik, 31);
        uint32_t offs[CELLS_WPT];
        x = x0; y = y0; w = w0;
#pragma unroll
        for (int k = 0; k < CELLS_WPT; ++k) {
            offs[k] = uint32_t(a);
            if (act[k]) {
                uint32_t cw8[8], qz, qy, qx;
                quad_word_act(g, p.NWg, p.NWc, q, k, x, y, w, cw8);
                owned_quads(g, cw8, act[k], x, y, w, qz, qy, qx);
                uint32_t ex[12];
                if (want_k) {
#pragma unroll
                    for (int e = 0; e < 12; ++e) ex[e] = cw8[iso_edge_corner(2 * e)] ^ cw8[iso_edge_corner(2 * e + 1)];
                }
                const uint32_t row = (uint32_t(x) * uint32_t(g.ny - 1) + uint32_t(y)) * uint32_t(g.nz - 1) + 32u * w;
                uint32_t m = act[k];
                while (m) {
                    const int b = __ffs(m) - 1;
                    m &= m - 1;
                    const uint32_t oz = (qz >> b) & 1u, oy = (qy >> b) & 1u, ox = (qx >> b) & 1u;
                    if (a < cap) {
                        cell_ids[a] = row + b;
                        qoff[a] = uint32_t(qq);
                        qbits[a] = uint8_t(oz | (oy << 1) | (ox << 2) | (((cw8[0] >> b) & 1u) << 3));
                        if (want_k) cell_off[a] = uint32_t(kk);
                    }
                    qq += oz + oy + ox;
                    if (want_k) kk += cell_crossings(ex, b);
                    ++a;
                }
            }
            next_point_word(g, p.NWg, x, y, w);
        }
        if (pw < p.PW) store_masks(offA, pw, p.PW, offs);
    }
}

// Active index of cell (cx, cy, cz) from the point-word masks and prefixes of
// dc_cells.
__device__ __forceinline__ uint32_t active_index_pw(const uint32_t* actm, const uint32_t* offA, const Grid3& g,
                                                    int cx, int cy, int cz) {
    const int NWg = (g.nz + 31) / 32;
    const long long wi = ((long long)cx * g.ny + cy) * NWg + (cz >> 5);
    return offA[wi] + __popc(actm[wi] & ((1u << (cz & 31)) - 1u));
}

// Cells along one axis whose closed interval [coord(i), coord(i + 1)] holds v,
// for v in cell c's interval: [i0, i1] around c (wider than c +- 1 only when
// grid coordinates repeat, on grids finer than FP32 resolves).
__device__ __forceinline__ void cells_holding(const Grid3& g, int axis, int c, float v, int& i0, int& i1) {
    const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    i0 = c;
    i1 = c;
    while (i0 > 0 && coord(g, axis, uint32_t(i0)) == v) --i0;
    while (i1 < n - 2 && coord(g, axis, uint32_t(i1 + 1)) == v) ++i1;
}

// Representative of used cell a whose vertex p lies on a face of its box: the
// smallest index among the used cells around that face with the same position.
__device__ __noinline__ uint32_t face_rep(const Grid3& g, uint32_t a, uint32_t cid, float px, float py, float pz,
                                          const uint8_t* __restrict__ used, const float* __restrict__ dual,
                                          const uint32_t* __restrict__ actm, const uint32_t* __restrict__ offA) {
    const float p[3] = {px, py, pz};
    const int cz = int(cid % uint32_t(g.nz - 1));
    const uint32_t rr = cid / uint32_t(g.nz - 1);
    const int cy = int(rr % uint32_t(g.ny - 1)), cx = int(rr / uint32_t(g.ny - 1));
    int x0, x1, y0, y1, z0, z1;
    cells_holding(g, 0, cx, p[0], x0, x1);
    cells_holding(g, 1, cy, p[1], y0, y1);
    cells_holding(g, 2, cz, p[2], z0, z1);
    const int NWg = (g.nz + 31) / 32;
    const uint32_t k0 = pos_bits(p[0]), k1 = pos_bits(p[1]), k2 = pos_bits(p[2]);
    uint32_t rep = a;
    for (int x = x0; x <= x1; ++x)
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) {
                if (x == cx && y == cy && z == cz) continue;
                const long long wi = ((long long)x * g.ny + y) * NWg + (z >> 5);  // point word
                const uint32_t mw = actm[wi], bit = uint32_t(z & 31);
                if (!((mw >> bit) & 1u)) continue;
                const uint32_t ib = offA[wi] + __popc(mw & ((1u << bit) - 1u));
                if (ib < rep && used[ib] && pos_bits(dual[3ll * ib]) == k0 && pos_bits(dual[3ll * ib + 1]) == k1 &&
                    pos_bits(dual[3ll * ib + 2]) == k2)
                    rep = ib;
            }
    return rep;
}

// Weld, step 1 (one thread per active cell): vmap[a] = 0xffffffff when no face
// uses the cell, 0 when its vertex is a representative (numbered in step 3),
// else 0x80000000 | its representative; representatives per block of DC_BLOCK
// cells into blk.
__global__ void __launch_bounds__(DC_BLOCK) dc_weld_flags(Grid3 g, const uint32_t* __restrict__ cell_ids,
                                                          const uint8_t* __restrict__ used,
                                                          const float* __restrict__ dual,
                                                          const uint32_t* __restrict__ actm,
                                                          const uint32_t* __restrict__ offA,
                                                          const long long* __restrict__ eff,
                                                          uint32_t* __restrict__ vmap,
                                                          unsigned long long* __restrict__ blk) {
    __shared__ uint32_t sm[66];
    iso::grid_wait();
    const long long a = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    const long long A = eff[0];
    uint32_t is = 0;
    if (a < A) {
        const uint32_t u = used[a];
        uint32_t m = 0xffffffffu;
        if (u) {
            uint32_t rep = uint32_t(a);
            if (u & 2u) rep = face_rep(g, rep, cell_ids[a], dual[3 * a], dual[3 * a + 1], dual[3 * a + 2], used, dual,
                                       actm, offA);
            is = rep == uint32_t(a) ? 1u : 0u;
            m = is ? 0u : (0x80000000u | rep);
        }
        vmap[a] = m;
    }
    uint32_t e0, e1, t0, t1;
    block_scan2(is, 0u, e0, e1, t0, t1, sm);
    if (threadIdx.x == 0) {
        blk[2 * blockIdx.x] = t0;
        blk[2 * blockIdx.x + 1] = 0;
    }
}

// Weld, step 3: representatives numbered in cell order (block offsets from the
// scan of step 2), their positions (and source cells) written.
__global__ void __launch_bounds__(DC_BLOCK) dc_weld_number(const float* __restrict__ dual,
                                                           const long long* __restrict__ eff,
                                                           const unsigned long long* __restrict__ blk,
                                                           const long long* __restrict__ vtot,
                                                           uint32_t* __restrict__ vmap, float* __restrict__ vout,
                                                           uint32_t* __restrict__ vsrc, long long* counts) {
    __shared__ uint32_t sm[66];
    iso::grid_wait();
    const long long a = (long long)blockIdx.x * DC_BLOCK + threadIdx.x;
    const long long A = eff[0];
    const uint32_t is = (a < A && vmap[a] == 0u) ? 1u : 0u;
    uint32_t e0, e1, t0, t1;
    block_scan2(is, 0u, e0, e1, t0, t1, sm);
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[0] = vtot[0];
    if (!is) return;
    const unsigned long long o = blk[2 * blockIdx.x] + e0;  // < V <= A: inside the vertex capacity
    vmap[a] = uint32_t(o);
    vout[3 * o] = dual[3 * a];
    vout[3 * o + 1] = dual[3 * a + 1];
    vout[3 * o + 2] = dual[3 * a + 2];
    if (vsrc) vsrc[o] = uint32_t(a);
}

// Final vertex number of active cell i: its own, or its representative's.
__device__ __forceinline__ int32_t vertex_of(const uint32_t* vmap, uint32_t i) {
    uint32_t m = vmap[i];
    if (m != 0xffffffffu && (m & 0x80000000u)) m = vmap[m & 0x7fffffffu];
    return int32_t(m);
}

// The quads active cell a owns, in the reference's order and orientation
// (src/dc.cu:101-157): the 4 cells around the edge are p - o_i with the offsets
// of edge_neighbors_table (src/shared_luts.cu:78-81), the owner being o_0 = 0.
__global__ void __launch_bounds__(256) dc_cell_quads(const uint8_t* __restrict__ qbits, Grid3 g,
                                                     const uint32_t* __restrict__ cell_ids,
                                                     const uint32_t* __restrict__ qoff,
                                                     const uint32_t* __restrict__ actm,
                                                     const uint32_t* __restrict__ offA,
                                                     const float* __restrict__ dual,
                                                     const uint32_t* __restrict__ vmap,
                                                     const long long* __restrict__ eff, int32_t* __restrict__ faces) {
    iso::grid_wait();
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= eff[0]) return;
    const uint32_t cid = cell_ids[a];
    const int cz = int(cid % uint32_t(g.nz - 1));
    const uint32_t rr = cid / uint32_t(g.nz - 1);
    const int cy = int(rr % uint32_t(g.ny - 1)), cx = int(rr / uint32_t(g.ny - 1));
    // owned edges (z, y, x) and the sign of the low corner, from dc_cells_write
    const uint32_t qb = qbits[a];
    const bool ez = qb & 1u, ey = qb & 2u, ex = qb & 4u;
    const uint32_t s0 = (qb >> 3) & 1u;
    if (!(qb & 7u)) return;
    unsigned long long q = qoff[a];
    const float own[3] = {dual[3 * a], dual[3 * a + 1], dual[3 * a + 2]};
#pragma unroll
    for (int ax = 2; ax >= 0; --ax) {
        if (!(ax == 2 ? ez : (ax == 1 ? ey : ex))) continue;
        // offsets o_1..o_3 of the other three cells
        int o[3][3];
        if (ax == 0) {
            const int t[3][3] = {{0, 1, 0}, {0, 1, 1}, {0, 0, 1}};
            for (int u = 0; u < 3; ++u) for (int d = 0; d < 3; ++d) o[u][d] = t[u][d];
        } else if (ax == 1) {
            const int t[3][3] = {{0, 0, 1}, {1, 0, 1}, {1, 0, 0}};
            for (int u = 0; u < 3; ++u) for (int d = 0; d < 3; ++d) o[u][d] = t[u][d];
        } else {
            const int t[3][3] = {{1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
            for (int u = 0; u < 3; ++u) for (int d = 0; d < 3; ++d) o[u][d] = t[u][d];
        }
        uint32_t qi[4];
        qi[0] = uint32_t(a);
#pragma unroll
        for (int u = 0; u < 3; ++u)
            qi[u + 1] = active_index_pw(actm, offA, g, cx - o[u][0], cy - o[u][1], cz - o[u][2]);
        // is_out = v(p0) <= v(p1): for a crossed edge, p0 below the level
        if (!s0) {
            const uint32_t t0 = qi[0], t1 = qi[1];
            qi[0] = qi[3]; qi[1] = qi[2]; qi[2] = t1; qi[3] = t0;
        }
        float v[4][3];
#pragma unroll
        for (int t = 0; t < 4; ++t)
#pragma unroll
            for (int d = 0; d < 3; ++d) v[t][d] = qi[t] == uint32_t(a) ? own[d] : dual[3ll * qi[t] + d];
        int32_t f[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) f[t] = vertex_of(vmap, qi[t]);
        int32_t* o6 = faces + 6 * q;
        if (dist3(v[0], v[2], g.fma) > dist3(v[1], v[3], g.fma)) {
            o6[0] = f[1]; o6[1] = f[3]; o6[2] = f[0];
            o6[3] = f[3]; o6[4] = f[1]; o6[5] = f[2];
        } else {
            o6[0] = f[2]; o6[1] = f[0]; o6[2] = f[1];
            o6[3] = f[0]; o6[4] = f[2]; o6[5] = f[3];
        }
        ++q;
    }
}

}  // namespace

// mc_signs lives in mc_dense.cu
#include "mc_dense.cuh"

// ---------------------------------------------------------------------------
// C ABI

// Exclusive scan of per-block (u64, u64) sums in place, totals -> totals[0..1]
// (used by the sparse-grid kernels).
void iso_block_scan_launch(unsigned long long* blk, long long nblk, long long* totals, cudaStream_t st) {
    dc_block_scan<<<1, 1024, 0, st>>>(blk, nblk, totals);
}

extern "C" {

size_t iso_dc_workspace_size(int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2) return 256;
    const long long NWg = (nz + 31) / 32, NWc = (nz - 1 + 31) / 32;
    const long long cwords = (long long)(nx - 1) * (ny - 1) * NWc;
    const long long pwords = (long long)nx * ny * NWg;
    const long long nblk = (std::max(cwords, pwords) + DC_BLOCK - 1) / DC_BLOCK;
    size_t o = 0;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    o = al(o + size_t(pwords) * 4);       // signs
    o = al(o + size_t(std::max(cwords, pwords)) * 4);  // active masks (by cell word, or by point word)
    o = al(o + size_t(std::max(cwords, pwords)) * 4);  // active prefixes
    o = al(o + size_t(nblk) * 16);        // cell block sums
    o = al(o + size_t(nblk) * 16);        // quad block sums
    return o + 1024;
}

}  // extern "C"

namespace {
struct DcWs {
    uint32_t *S, *actm, *offA;
    unsigned long long *blkC, *blkQ;
    long long cwords, pwords, nblkC, nblkQ;
};
DcWs carve(void* ws, int nx, int ny, int nz) {
    DcWs w;
    const long long NWg = (nz + 31) / 32, NWc = (nz - 1 + 31) / 32;
    w.cwords = (long long)(nx - 1) * (ny - 1) * NWc;
    w.pwords = (long long)nx * ny * NWg;
    w.nblkC = (w.cwords + DC_BLOCK - 1) / DC_BLOCK;
    w.nblkQ = (w.pwords + DC_BLOCK - 1) / DC_BLOCK;
    const long long nblk = std::max(w.nblkC, w.nblkQ);
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    w.S = reinterpret_cast<uint32_t*>(b + o);    o = al(o + size_t(w.pwords) * 4);
    const size_t nmask = size_t(std::max(w.cwords, w.pwords));
    w.actm = reinterpret_cast<uint32_t*>(b + o); o = al(o + nmask * 4);
    w.offA = reinterpret_cast<uint32_t*>(b + o); o = al(o + nmask * 4);
    w.blkC = reinterpret_cast<unsigned long long*>(b + o); o = al(o + size_t(nblk) * 16);
    w.blkQ = reinterpret_cast<unsigned long long*>(b + o);
    return w;
}
}  // namespace

extern "C" {

int iso_dc_classify(const float* values, int nx, int ny, int nz, float level, void* ws, size_t ws_bytes,
                    long long* counts, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    if (ws_bytes < iso_dc_workspace_size(nx, ny, nz)) return iso::fail_code(ISO_ERR_WORKSPACE);
    DcWs w = carve(ws, nx, ny, nz);
    const float amin[3] = {0, 0, 0}, amax[3] = {1, 1, 1};
    Grid3 g = make_grid(nx, ny, nz, amin, amax);
    {
        iso::ProfScope ps("mc_signs", st);
        mc_signs_launch(values, nx, ny, nz, level, w.S, st);
    }
    iso::ProfScope ps("dc_classify", st, 2);
    dc_cell_count<<<blocks_for(w.cwords, DC_BLOCK), DC_BLOCK, 0, st>>>(w.S, g, w.cwords, w.blkC);
    dc_block_scan<<<1, 1024, 0, st>>>(w.blkC, w.nblkC, counts);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_intersect(const float* values, int nx, int ny, int nz, const float* aabb_min,
                     const float* aabb_max, float level, void* ws, long long A, long long K, float* points,
                     float* normals, int* cell_ids, int* cell_offsets, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    DcWs w = carve(ws, nx, ny, nz);
    Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    iso::ProfScope ps("dc_intersect", st, A > 0 && points ? 2 : 1);
    dc_intersect<<<blocks_for(w.cwords, DC_BLOCK), DC_BLOCK, 0, st>>>(
        values, w.S, g, level, w.cwords, w.blkC, w.actm, w.offA, points, normals,
        reinterpret_cast<uint32_t*>(cell_ids), reinterpret_cast<uint32_t*>(cell_offsets), A, K, nullptr);
    if (A == 0 && cell_offsets) cudaMemsetAsync(cell_offsets, 0, 4, st);
    if (A > 0 && points)
        dc_points<<<blocks_for(A, iso::tune_get(iso::TUNE_DC_CELL_THREADS)), iso::tune_get(iso::TUNE_DC_CELL_THREADS), 0,
                    st>>>(values, g, level, reinterpret_cast<uint32_t*>(cell_ids),
                                                      reinterpret_cast<uint32_t*>(cell_offsets), A, points,
                                                      normals);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

// Active cells, their crossing offsets and the dual vertices, without writing
// crossing points or normals (dual_contouring without a caller intersection).
int iso_dc_intersect_solve(const float* values, int nx, int ny, int nz, const float* aabb_min,
                           const float* aabb_max, float level, void* ws, long long A, long long K,
                           int* cell_ids, int* cell_offsets, float reg, float svd_tol, float* dual, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2 || A <= 0) return 0;
    if (!cell_ids || !cell_offsets || !dual) return iso::fail_code(ISO_ERR_ARG);
    DcWs w = carve(ws, nx, ny, nz);
    Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    {
        iso::ProfScope ps("dc_intersect", st);
        dc_intersect<<<blocks_for(w.cwords, DC_BLOCK), DC_BLOCK, 0, st>>>(
            values, w.S, g, level, w.cwords, w.blkC, w.actm, w.offA, nullptr, nullptr,
            reinterpret_cast<uint32_t*>(cell_ids), reinterpret_cast<uint32_t*>(cell_offsets), A, K, nullptr);
    }
    iso::ProfScope ps("dc_solve", st);
    const int bt = iso::tune_get(iso::TUNE_DC_CELL_THREADS);
    solve_kernel(g)<<<blocks_for(A, bt), bt, 0, st>>>(values, g, level, reinterpret_cast<uint32_t*>(cell_ids), A, reg,
                                                    svd_tol, dual, nullptr, nullptr, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_normals(const float* values, int nx, int ny, int nz, const float* aabb_min,
                   const float* aabb_max, const float* points, const int* cell_ids,
                   const int* cell_offsets, long long A, float* normals, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A <= 0) return 0;
    Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    iso::ProfScope ps("dc_normals", st);
    dc_normals<<<blocks_for(A, 256), 256, 0, st>>>(values, g, points,
                                                   reinterpret_cast<const uint32_t*>(cell_ids),
                                                   reinterpret_cast<const uint32_t*>(cell_offsets), A,
                                                   normals);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_solve(int nx, int ny, int nz, const float* aabb_min, const float* aabb_max, const float* points,
                 const float* normals, const int* cell_ids, const int* cell_offsets, long long A, float reg,
                 float svd_tol, float* dual, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A <= 0) return 0;
    Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    iso::ProfScope ps("dc_solve", st);
    const int bt = iso::tune_get(iso::TUNE_DC_CELL_THREADS);
    dc_solve<<<blocks_for(A, bt), bt, 0, st>>>(points, normals, reinterpret_cast<const uint32_t*>(cell_ids),
                                                 reinterpret_cast<const uint32_t*>(cell_offsets), A, g, reg,
                                                 svd_tol, dual);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

// Active masks and prefixes only (when the intersection was made earlier).
int iso_dc_cells(const float* values, int nx, int ny, int nz, float level, void* ws, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    DcWs w = carve(ws, nx, ny, nz);
    const float amin[3] = {0, 0, 0}, amax[3] = {1, 1, 1};
    Grid3 g = make_grid(nx, ny, nz, amin, amax);
    iso::ProfScope ps("dc_intersect", st);
    dc_intersect<<<blocks_for(w.cwords, DC_BLOCK), DC_BLOCK, 0, st>>>(
        values, w.S, g, level, w.cwords, w.blkC, w.actm, w.offA, nullptr, nullptr, nullptr, nullptr, -1, 0, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_quads_count(int nx, int ny, int nz, void* ws, long long* counts, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    DcWs w = carve(ws, nx, ny, nz);
    const float amin[3] = {0, 0, 0}, amax[3] = {1, 1, 1};
    Grid3 g = make_grid(nx, ny, nz, amin, amax);
    iso::ProfScope ps("dc_quads", st, 2);
    dc_quad_count<<<blocks_for(w.pwords, DC_BLOCK), DC_BLOCK, 0, st>>>(w.S, g, w.pwords, w.blkQ);
    dc_block_scan<<<1, 1024, 0, st>>>(w.blkQ, w.nblkQ, counts);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_quads_emit(int nx, int ny, int nz, void* ws, const float* dual, int* tri, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    DcWs w = carve(ws, nx, ny, nz);
    const float amin[3] = {0, 0, 0}, amax[3] = {1, 1, 1};
    Grid3 g = make_grid(nx, ny, nz, amin, amax);
    iso::ProfScope ps("dc_quads", st);
    dc_quad_emit<<<blocks_for(w.pwords, DC_BLOCK), DC_BLOCK, 0, st>>>(w.S, g, w.pwords, w.blkQ, w.actm,
                                                                     w.offA, dual, tri, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

size_t iso_dc_weld_workspace_size(long long A) {
    uint32_t cap = 1024;
    while ((long long)cap < 2 * A + 1024) cap <<= 1;
    const long long nblk = (A + DC_BLOCK - 1) / DC_BLOCK + 1;
    return size_t(A) * 12 + size_t(cap) * 4 + size_t(nblk) * 16 + 4096;
}

// Weld step 1: used marks, hash, representatives; counts[0] <- V.
int iso_dc_weld_count(const float* dual, long long A, const int* tri, long long ntri, void* ws,
                      size_t ws_bytes, long long* counts, int* status, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (ws_bytes < iso_dc_weld_workspace_size(A)) return iso::fail_code(ISO_ERR_WORKSPACE);
    uint32_t cap = 1024;
    while ((long long)cap < 2 * A + 1024) cap <<= 1;
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    uint32_t* used = reinterpret_cast<uint32_t*>(b);
    uint32_t* rep = used + A;
    uint32_t* newidx = rep + A;
    uint32_t* table = newidx + A;
    unsigned long long* blk = reinterpret_cast<unsigned long long*>(
        (reinterpret_cast<uintptr_t>(table + cap) + 15) & ~uintptr_t(15));
    const long long nblk = (A + DC_BLOCK - 1) / DC_BLOCK;
    iso::ProfScope ps("dc_weld", st, (ntri > 0 ? 1 : 0) + (A > 0 ? 4 : 0));
    cudaMemsetAsync(used, 0, size_t(A) * 4, st);
    cudaMemsetAsync(table, 0xff, size_t(cap) * 4, st);
    if (ntri > 0) dc_mark_used<<<blocks_for(ntri, 256), 256, 0, st>>>(tri, ntri, used, nullptr);
    if (A > 0) {
        dc_hash_insert<<<blocks_for(A, 256), 256, 0, st>>>(dual, used, A, table, cap - 1, status, nullptr);
        dc_hash_lookup<<<blocks_for(A, 256), 256, 0, st>>>(dual, used, A, table, cap - 1, rep, nullptr);
        dc_rep_count<<<unsigned(nblk), DC_BLOCK, 0, st>>>(rep, A, blk, nullptr);
        dc_block_scan<<<1, 1024, 0, st>>>(blk, nblk, counts);
    } else {
        cudaMemsetAsync(counts, 0, 16, st);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

// Weld step 2: write vertices [V, 3] and faces [ntri / 3, 3]; vertex_source
// (optional, [V]) receives the dual vertex (active cell) each vertex came from.
int iso_dc_weld_write_src(const float* dual, long long A, const int* tri, long long ntri, void* ws,
                          float* vout, int* fout, int* vertex_source, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t cap = 1024;
    while ((long long)cap < 2 * A + 1024) cap <<= 1;
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    uint32_t* used = reinterpret_cast<uint32_t*>(b);
    uint32_t* rep = used + A;
    uint32_t* newidx = rep + A;
    uint32_t* table = newidx + A;
    unsigned long long* blk = reinterpret_cast<unsigned long long*>(
        (reinterpret_cast<uintptr_t>(table + cap) + 15) & ~uintptr_t(15));
    const long long nblk = (A + DC_BLOCK - 1) / DC_BLOCK;
    iso::ProfScope ps("dc_weld", st, (A > 0 ? 1 : 0) + (ntri > 0 ? 1 : 0));
    if (A > 0)
        dc_rep_write<<<unsigned(nblk), DC_BLOCK, 0, st>>>(rep, A, blk, dual, newidx, vout,
                                                           reinterpret_cast<uint32_t*>(vertex_source), nullptr);
    if (ntri > 0) dc_remap<<<blocks_for(ntri, 256), 256, 0, st>>>(tri, ntri, rep, newidx, fout, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_weld_write(const float* dual, long long A, const int* tri, long long ntri, void* ws,
                      float* vout, int* fout, void* stream) {
    return iso_dc_weld_write_src(dual, A, tri, ntri, ws, vout, fout, nullptr, stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// One call, no host synchronisation: for stream capture and for callers that
// size their buffers once.  Capacities: vertex_capacity bounds the active cells
// (dual vertices before the weld, A >= V), face_capacity the faces (2 per quad).

namespace {
struct DcDenseWs {
    DcWs d;
    unsigned long long* zero;  // cleared by the sign pass
    long long nzero;
    long long* misc;           // [0..1] V  [4..7] eff
    unsigned long long* wblk;  // weld: representatives per block of DC_BLOCK cells
    uint32_t *wsum, *csum;     // dc_cells: 4 words per warp, per CTA
    long long ntC, ntV;        // CTAs of the dc_cells kernels and of the weld
    uint32_t *cells, *qoff, *vmap;
    uint8_t *used, *qbits;
    float* dual;
    float* gc;  // grid coordinates, x then y then z
    size_t total;
};

DcDenseWs carve_dense(void* ws, int nx, int ny, int nz, long long capA) {
    DcDenseWs w{};
    const size_t base = iso_dc_workspace_size(nx, ny, nz);
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    if (ws) w.d = carve(b, nx, ny, nz);
    const long long pwords = (long long)nx * ny * ((nz + 31) / 32);
    w.ntC = (pwords + CELLS_TILE - 1) / CELLS_TILE;
    w.ntV = (capA + DC_BLOCK - 1) / DC_BLOCK;
    size_t o = (base + 255) & ~size_t(255);
    auto take = [&](size_t bytes) {
        uint8_t* p = ws ? b + o : nullptr;
        o = (o + std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        return p;
    };
    w.nzero = 16;
    w.zero = reinterpret_cast<unsigned long long*>(take(size_t(w.nzero) * 8));
    w.misc = reinterpret_cast<long long*>(w.zero);
    w.wblk = reinterpret_cast<unsigned long long*>(take(size_t(w.ntV + 1) * 16));
    w.wsum = reinterpret_cast<uint32_t*>(take(size_t(w.ntC) * CELLS_WARPS * 16));
    w.csum = reinterpret_cast<uint32_t*>(take(size_t(w.ntC) * 16));
    w.cells = reinterpret_cast<uint32_t*>(take(size_t(capA) * 4));
    w.qoff = reinterpret_cast<uint32_t*>(take(size_t(capA) * 4));
    w.vmap = reinterpret_cast<uint32_t*>(take(size_t(capA) * 4));
    w.used = take(size_t(capA));
    w.qbits = take(size_t(capA));
    w.dual = reinterpret_cast<float*>(take(size_t(capA) * 12));
    w.gc = reinterpret_cast<float*>(take(size_t(nx + ny + nz) * 4));
    w.total = o + 256;
    return w;
}
}  // namespace

extern "C" {

size_t iso_dc_dense_workspace_size(int nx, int ny, int nz, long long vertex_capacity, long long face_capacity) {
    if (nx < 2 || ny < 2 || nz < 2) return 256;
    if (vertex_capacity < 0 || face_capacity < 0) return 0;
    return carve_dense(nullptr, nx, ny, nz, vertex_capacity).total;
}

int iso_dc_dense_ex(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                    float level, float reg, float svd_tol, float* vertices, long long vertex_capacity, int* faces,
                    long long face_capacity, void* workspace, size_t workspace_bytes, long long* counts, int* status,
                    int* cell_ids, int* cell_offsets, int* vertex_source, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!counts || !status || !aabb_min || !aabb_max || vertex_capacity < 0 || face_capacity < 0) return iso::fail_code(ISO_ERR_ARG);
    if ((long long)nx * ny * nz > 0x7fffffffll) return iso::fail_code(ISO_ERR_ARG);
    if (nx < 2 || ny < 2 || nz < 2)
        return cudaMemsetAsync(counts, 0, 5 * sizeof(long long), st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    if (!values || (vertex_capacity && !vertices) || (face_capacity && !faces)) return iso::fail_code(ISO_ERR_ARG);
    const long long capA = vertex_capacity, capQ = face_capacity / 2;
    if (workspace_bytes < iso_dc_dense_workspace_size(nx, ny, nz, vertex_capacity, face_capacity))
        return iso::fail_code(ISO_ERR_WORKSPACE);
    const DcDenseWs w = carve_dense(workspace, nx, ny, nz, capA);
    const Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    long long* eff = w.misc + 4;
    uint32_t* cells = cell_ids ? reinterpret_cast<uint32_t*>(cell_ids) : w.cells;
    {
        iso::ProfScope ps("mc_signs", st);
        mc_signs_launch(values, nx, ny, nz, level, w.d.S, st, w.zero, w.nzero);
    }
    {
        iso::ProfScope ps("dc_classify", st, 3);
        const uint32_t* S = w.d.S;
        iso::launch_pdl(dc_cells_count, unsigned(w.ntC), unsigned(CELLS_THREADS), st, S, g, w.d.actm, w.wsum,
                        w.csum, w.gc);
        iso::launch_pdl(dc_cells_scan, 1u, 1024u, st, w.csum, w.ntC, capA, capQ, eff, counts,
                        reinterpret_cast<uint32_t*>(cell_offsets), status);
        iso::launch_pdl(dc_cells_write, unsigned(w.ntC), unsigned(CELLS_THREADS), st, S, g,
                        static_cast<const uint32_t*>(w.d.actm), static_cast<const uint32_t*>(w.wsum),
                        static_cast<const uint32_t*>(w.csum), w.d.offA, cells, w.qoff, w.qbits,
                        reinterpret_cast<uint32_t*>(cell_offsets), capA);
    }
    if (capA > 0) {
        {
            iso::ProfScope ps("dc_solve", st);
            const int bt = iso::tune_get(iso::TUNE_DC_CELL_THREADS);
            iso::launch_pdl(solve_kernel(g), blocks_for(capA, bt), unsigned(bt), st, values, g, level,
                            static_cast<const uint32_t*>(cells), capA, reg, svd_tol, w.dual,
                            static_cast<const long long*>(eff), w.used, static_cast<const float*>(w.gc));
        }
        {
            iso::ProfScope ps("dc_weld", st, 3);
            iso::launch_pdl(dc_weld_flags, unsigned(w.ntV), unsigned(DC_BLOCK), st, g,
                            static_cast<const uint32_t*>(cells), static_cast<const uint8_t*>(w.used),
                            static_cast<const float*>(w.dual), static_cast<const uint32_t*>(w.d.actm),
                            static_cast<const uint32_t*>(w.d.offA), static_cast<const long long*>(eff), w.vmap,
                            w.wblk);
            iso::launch_pdl(dc_block_scan, 1u, 1024u, st, w.wblk, w.ntV, w.misc);
            iso::launch_pdl(dc_weld_number, unsigned(w.ntV), unsigned(DC_BLOCK), st,
                            static_cast<const float*>(w.dual), static_cast<const long long*>(eff),
                            static_cast<const unsigned long long*>(w.wblk), static_cast<const long long*>(w.misc),
                            w.vmap, vertices, reinterpret_cast<uint32_t*>(vertex_source), counts);
        }
        {
            iso::ProfScope ps("dc_quads", st);
            iso::launch_pdl(dc_cell_quads, blocks_for(capA, 256), 256u, st, static_cast<const uint8_t*>(w.qbits), g,
                            static_cast<const uint32_t*>(cells), static_cast<const uint32_t*>(w.qoff),
                            static_cast<const uint32_t*>(w.d.actm), static_cast<const uint32_t*>(w.d.offA),
                            static_cast<const float*>(w.dual), static_cast<const uint32_t*>(w.vmap),
                            static_cast<const long long*>(eff), faces);
        }
    }
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_dense(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                 float level, float reg, float svd_tol, float* vertices, long long vertex_capacity, int* faces,
                 long long face_capacity, void* workspace, size_t workspace_bytes, long long* counts, int* status,
                 void* stream) {
    return iso_dc_dense_ex(values, nx, ny, nz, aabb_min, aabb_max, level, reg, svd_tol, vertices, vertex_capacity,
                           faces, face_capacity, workspace, workspace_bytes, counts, status, nullptr, nullptr, nullptr,
                           stream);
}

}  // extern "C"
