// SparseGrid extraction on sm_103a (isoext src/grid/sparse.cu, src/mc/mc.cu).
//
// A sparse grid is a sorted list of cell ids over the (n-1)^3 cell lattice with
// its own 8 corner values per cell ([N, 8], Morton corner order).  Cells share
// no storage, so isoext welds vertices by exact position (src/utils.cu:32-59);
// so does this path (hash weld in dc_dense.cu), which keeps it exact even when
// two cells disagree about a shared corner's value.
//
//   mc_count / mc_emit   per cell: case, edge lerps, triangles whose three
//                        positions differ (src/mc/nagae.cu:34-80), written as a
//                        triangle soup in cell order.
//   its_count / its_emit per active cell: crossings in edge-bit order, normals
//                        (src/its.cu:37-90, 186-268).
//   quads                each cell's x/y/z edges at its lowest corner, in cell
//                        order = isoext's (p0, axis) quad order; a quad needs its
//                        4 cells in the grid (binary search) and active.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "mc_dense.cuh"
#include "profile.cuh"

namespace {

constexpr int SP_BLOCK = 256;  // per-cell state is ~70 registers

struct SpGrid {
    int nx, ny, nz;
    float amin[3], asize[3];
    float level;
    int method;
    float tau;  // edge parameters within tau of 0 or 1 may put two vertices on one position
    bool fma;   // arithmetic reading (iso::arith_fma at the call)
};

__device__ __forceinline__ void cell_xyz(const SpGrid& g, uint32_t id, int& x, int& y, int& z) {
    z = int(id % uint32_t(g.nz - 1));
    const uint32_t r = id / uint32_t(g.nz - 1);
    y = int(r % uint32_t(g.ny - 1));
    x = int(r / uint32_t(g.ny - 1));
}

struct Cell8 {
    float v[8];
    float p[8][3];
    bool fma;  // the grid's arithmetic reading (set with the positions)
};

// The 8 values of cell c (two 16-byte loads).
__device__ __forceinline__ void load_vals(const float* vals, long long c, Cell8& cc) {
    const float4* v4 = reinterpret_cast<const float4*>(vals + 8 * c);
    const float4 a = __ldg(v4), b = __ldg(v4 + 1);
    cc.v[0] = a.x; cc.v[1] = a.y; cc.v[2] = a.z; cc.v[3] = a.w;
    cc.v[4] = b.x; cc.v[5] = b.y; cc.v[6] = b.z; cc.v[7] = b.w;
}

// Corner positions of cell (x, y, z) (include/utils.cuh:62-80).
__device__ __forceinline__ void set_coords(const SpGrid& g, int x, int y, int z, Cell8& cc) {
    const float cx0 = iso::grid_coord(x, g.nx, g.amin[0], g.asize[0], g.fma);
    const float cx1 = iso::grid_coord(x + 1, g.nx, g.amin[0], g.asize[0], g.fma);
    const float cy0 = iso::grid_coord(y, g.ny, g.amin[1], g.asize[1], g.fma);
    const float cy1 = iso::grid_coord(y + 1, g.ny, g.amin[1], g.asize[1], g.fma);
    const float cz0 = iso::grid_coord(z, g.nz, g.amin[2], g.asize[2], g.fma);
    const float cz1 = iso::grid_coord(z + 1, g.nz, g.amin[2], g.asize[2], g.fma);
    cc.fma = g.fma;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        cc.p[k][0] = (k >> 2) ? cx1 : cx0;
        cc.p[k][1] = ((k >> 1) & 1) ? cy1 : cy0;
        cc.p[k][2] = (k & 1) ? cz1 : cz0;
    }
}

__device__ __forceinline__ void load_cell(const SpGrid& g, const int* ids, const float* vals, long long c,
                                          Cell8& cc, int& x, int& y, int& z) {
    cell_xyz(g, uint32_t(ids[c]), x, y, z);
    load_vals(vals, c, cc);
    set_coords(g, x, y, z, cc);
}

// Values and case of cell c; positions only for a cell the surface crosses
// (most cells of a band are empty).
__device__ __forceinline__ uint32_t load_active(const SpGrid& g, const int* ids, const float* vals, long long c,
                                                Cell8& cc) {
    load_vals(vals, c, cc);
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) cs |= (iso::below(cc.v[k], g.level) ? 1u : 0u) << k;
    if (cs != 0 && cs != 255) {
        int x, y, z;
        cell_xyz(g, uint32_t(ids[c]), x, y, z);
        set_coords(g, x, y, z, cc);
    }
    return cs;
}

__device__ __forceinline__ uint32_t case_of(const Cell8& cc, float level) {
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) cs |= (iso::below(cc.v[k], level) ? 1u : 0u) << k;
    return cs;
}

__device__ __forceinline__ void edge_point(const Cell8& cc, int e, float level, float* p) {
    const int a = ISO_EDGE_CORNERS[2 * e], b = ISO_EDGE_CORNERS[2 * e + 1];
    const float t = iso::cross_t(level, cc.v[a], cc.v[b]);
#pragma unroll
    for (int q = 0; q < 3; ++q) p[q] = iso::lerp1(t, cc.p[a][q], cc.p[b][q], cc.fma);
}

__device__ __forceinline__ bool eq3(const float* a, const float* b) {
    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
}

__device__ __forceinline__ const signed char* tri_row(int method, uint32_t cs, int& ml) {
    if (method == 0) { ml = 15; return ISO_TRI_NAGAE + cs * 15; }
    ml = 12;
    return ISO_TRI_LORENSEN + cs * 12;
}

// Faces of one cell (positions of its crossed edges in ev).
__device__ __forceinline__ uint32_t mc_cell(const SpGrid& g, const Cell8& cc, float (*ev)[3]) {
    const uint32_t cs = case_of(cc, g.level);
    if (cs == 0 || cs == 255) return 0;
    const uint32_t est = ISO_EDGE_STATUS[cs];
#pragma unroll
    for (int e = 0; e < 12; ++e)
        if ((est >> e) & 1u) edge_point(cc, e, g.level, ev[e]);
    int ml;
    const signed char* tr = tri_row(g.method, cs, ml);
    uint32_t n = 0;
    for (int k = 0; k < ml && tr[k] >= 0; k += 3) {
        const float* a = ev[tr[k]];
        const float* b = ev[tr[k + 1]];
        const float* c = ev[tr[k + 2]];
        n += (!eq3(a, b) && !eq3(a, c) && !eq3(b, c));
    }
    return n;
}

__device__ __forceinline__ void block_scan1(uint32_t a, uint32_t& ea, uint32_t& ta, uint32_t* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t ia = a;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t x = __shfl_up_sync(~0u, ia, d);
        if (lane >= d) ia += x;
    }
    if (lane == 31) sm[warp] = ia;
    __syncthreads();
    if (warp == 0) {
        uint32_t x = lane < int(blockDim.x >> 5) ? sm[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, x, d);
            if (lane >= d) x += u;
        }
        sm[lane] = x;
    }
    __syncthreads();
    ea = (warp ? sm[warp - 1] : 0u) + ia - a;
    ta = sm[31];  // sum over all warps = block total
    __syncthreads();
}

// Faces of a crossed cell when no two of its vertices can share a position: all
// its crossed edges have t within [tau, 1 - tau], so no vertex comes within
// rounding of a corner (two edges' vertices can only meet there) and none of
// the case's triangles is degenerate.  Otherwise ~0u (count by positions).
__device__ __forceinline__ uint32_t mc_cell_fast(const SpGrid& g, const Cell8& cc, uint32_t cs) {
    bool near = false;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        const int a = iso_edge_corner(2 * e), b = iso_edge_corner(2 * e + 1);
        if ((((cs >> a) ^ (cs >> b)) & 1u) == 0u) continue;  // not crossed
        const float t = iso::cross_t(g.level, cc.v[a], cc.v[b]);
        near |= !(t >= g.tau && t <= 1.0f - g.tau);
    }
    return near ? ~0u : uint32_t(ISO_NTRI[g.method * 256 + cs]);
}

__global__ void __launch_bounds__(SP_BLOCK) sp_mc_count(SpGrid g, const int* __restrict__ ids,
                                                        const float* __restrict__ vals, long long n,
                                                        unsigned long long* blk) {
    __shared__ uint32_t sm[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t nf = 0;
    if (c < n) {
        Cell8 cc;
        load_vals(vals, c, cc);
        uint32_t cs = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) cs |= (iso::below(cc.v[k], g.level) ? 1u : 0u) << k;
        if (cs != 0 && cs != 255) {
            nf = mc_cell_fast(g, cc, cs);
            if (nf == ~0u) {  // a vertex near a corner: compare positions, as the emit pass does
                int x, y, z;
                cell_xyz(g, uint32_t(ids[c]), x, y, z);
                set_coords(g, x, y, z, cc);
                float ev[12][3];
                nf = mc_cell(g, cc, ev);
            }
        }
    }
    uint32_t e, t;
    block_scan1(nf, e, t, sm);
    if (threadIdx.x == 0) { blk[2 * blockIdx.x] = t; blk[2 * blockIdx.x + 1] = 0; }
}

__global__ void __launch_bounds__(SP_BLOCK) sp_mc_emit(SpGrid g, const int* __restrict__ ids,
                                                       const float* __restrict__ vals, long long n,
                                                       const unsigned long long* __restrict__ blk,
                                                       float* soup, const long long* __restrict__ dn) {
    __shared__ uint32_t sm[33];
    if (dn && dn[0] == 0) return;  // over capacity (or nothing to write): the sizes say so
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t nf = 0;
    Cell8 cc;
    float ev[12][3];
    uint32_t cs = 0;
    bool fast = false;
    if (c < n) {
        cs = load_active(g, ids, vals, c, cc);
        if (cs != 0 && cs != 255) {
            // the count pass's decision: far from corners every triangle of the case
            nf = mc_cell_fast(g, cc, cs);
            fast = nf != ~0u;
            if (fast) {
                const uint32_t est = ISO_EDGE_STATUS[cs];
#pragma unroll
                for (int q = 0; q < 12; ++q)
                    if ((est >> q) & 1u) edge_point(cc, q, g.level, ev[q]);
            } else {
                nf = mc_cell(g, cc, ev);
            }
        }
    }
    uint32_t e, t;
    block_scan1(nf, e, t, sm);
    if (!nf) return;
    unsigned long long f = blk[2 * blockIdx.x] + e;
    int ml;
    const signed char* tr = tri_row(g.method, cs, ml);
    for (int k = 0; k < ml && tr[k] >= 0; k += 3) {
        const float* a = ev[tr[k]];
        const float* b = ev[tr[k + 1]];
        const float* cpos = ev[tr[k + 2]];
        if (!fast && (eq3(a, b) || eq3(a, cpos) || eq3(b, cpos))) continue;
        float* o = soup + 9 * f;
        o[0] = a[0]; o[1] = a[1]; o[2] = a[2];
        o[3] = b[0]; o[4] = b[1]; o[5] = b[2];
        o[6] = cpos[0]; o[7] = cpos[1]; o[8] = cpos[2];
        ++f;
    }
}

// --- one-call sparse MC: crossed cells compacted per CTA ------------------------
//
// A CTA takes SP2_CHUNK consecutive cells.  It reads every cell's 8 values once
// for its case, compacts the crossed ones (a few percent of a band) into a list
// in shared memory, and does the per-crossed-cell work with full warps.  The
// emit writes each crossed cell's vertices once (the crossed edges its kept
// triangles use, in edge order) and the triangles as indices into that list, so
// the position weld hashes each distinct vertex about four times instead of
// six.

constexpr int SP2_THREADS = 256;
constexpr int SP2_ROUNDS = 16;                       // cells per thread
constexpr int SP2_CHUNK = SP2_THREADS * SP2_ROUNDS;  // cells per CTA

// Kept faces of crossed cell c (case cs) and the crossed edges they use
// (used).  Far from corners every triangle of the case is kept and every
// crossed edge used; otherwise the positions decide, as mc_cell does (ev then
// holds them).
__device__ __forceinline__ uint32_t sp_cell_summary(const SpGrid& g, const int* ids, long long c, Cell8& cc,
                                                    uint32_t cs, float (*ev)[3], uint32_t& used, bool& fast) {
    const uint32_t est = ISO_EDGE_STATUS[cs];
    uint32_t nf = mc_cell_fast(g, cc, cs);
    fast = nf != ~0u;
    if (fast) {
        used = est;
        return nf;
    }
    int x, y, z;
    cell_xyz(g, uint32_t(ids[c]), x, y, z);
    set_coords(g, x, y, z, cc);
#pragma unroll
    for (int e = 0; e < 12; ++e)
        if ((est >> e) & 1u) edge_point(cc, e, g.level, ev[e]);
    int ml;
    const signed char* tr = tri_row(g.method, cs, ml);
    used = 0;
    nf = 0;
    for (int k = 0; k < ml && tr[k] >= 0; k += 3) {
        const float* a = ev[tr[k]];
        const float* b = ev[tr[k + 1]];
        const float* d = ev[tr[k + 2]];
        if (eq3(a, b) || eq3(a, d) || eq3(b, d)) continue;
        used |= (1u << tr[k]) | (1u << tr[k + 1]) | (1u << tr[k + 2]);
        ++nf;
    }
    return nf;
}

__device__ __forceinline__ uint32_t sp_case(const SpGrid& g, const float* vals, long long c, Cell8& cc) {
    load_vals(vals, c, cc);
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) cs |= (iso::below(cc.v[k], g.level) ? 1u : 0u) << k;
    return cs;
}

// Block sum of two counts (thread 0 gets them).
__device__ __forceinline__ void sp_sum2(uint32_t& a, uint32_t& b, uint32_t (*sm)[SP2_THREADS / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        a += __shfl_xor_sync(~0u, a, d);
        b += __shfl_xor_sync(~0u, b, d);
    }
    if (lane == 0) { sm[0][warp] = a; sm[1][warp] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = 0;
        b = 0;
        for (int k = 0; k < SP2_THREADS / 32; ++k) { a += sm[0][k]; b += sm[1][k]; }
    }
}

// Ordered compaction of a chunk's crossed cells into list[] (cell order);
// returns their number.  The values are loaded four rounds at a time; each
// warp keeps its 16 ballots, and one barrier gives every list position.
__device__ __forceinline__ uint32_t sp_crossed(const SpGrid& g, const float* vals, long long n, long long c0,
                                               uint16_t* list, uint32_t (*wcnt)[SP2_THREADS / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t bal[SP2_ROUNDS];
#pragma unroll
    for (int r0 = 0; r0 < SP2_ROUNDS; r0 += 4) {
        float4 va[4], vb[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long c = c0 + (r0 + k) * SP2_THREADS + threadIdx.x;
            if (c < n) {
                const float4* v4 = reinterpret_cast<const float4*>(vals + 8 * c);
                va[k] = __ldg(v4);
                vb[k] = __ldg(v4 + 1);
            } else {
                va[k] = vb[k] = make_float4(g.level, g.level, g.level, g.level);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v[8] = {va[k].x, va[k].y, va[k].z, va[k].w, vb[k].x, vb[k].y, vb[k].z, vb[k].w};
            uint32_t cs = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) cs |= (iso::below(v[q], g.level) ? 1u : 0u) << q;
            bal[r0 + k] = __ballot_sync(~0u, cs != 0 && cs != 255);
        }
    }
    if (lane < SP2_ROUNDS) {  // wcnt holds [round][warp] counts (SP2_ROUNDS x warps)
        uint32_t mine = 0;
#pragma unroll
        for (int r = 0; r < SP2_ROUNDS; ++r)
            if (r == lane) mine = __popc(bal[r]);
        wcnt[lane][warp] = mine;
    }
    __syncthreads();
    uint32_t base = 0;
#pragma unroll
    for (int r = 0; r < SP2_ROUNDS; ++r) {
        uint32_t before = 0, all = 0;
#pragma unroll
        for (int k = 0; k < SP2_THREADS / 32; ++k) {
            const uint32_t c = wcnt[r][k];
            before += k < warp ? c : 0u;
            all += c;
        }
        if ((bal[r] >> lane) & 1u)
            list[base + before + __popc(bal[r] & ((1u << lane) - 1u))] = uint16_t(r * SP2_THREADS + threadIdx.x);
        base += all;
    }
    __syncthreads();  // wcnt is reused by the caller
    return base;
}

// Per crossed cell, what the emit needs in 32 bits: kept faces (bits 0-2),
// whether every triangle of the case is kept (3: no vertex near a corner),
// the crossed edges the kept triangles use (4-15), and for each edge an
// earlier cell of the same x may make (sp_slot), whose entry it takes (2 bits
// from bit 16 + 2 slot: 0 its own, 1 the z-neighbour's, 2 the y-neighbour's,
// 3 the diagonal (y - 1, z -+ 1) neighbour's; see sp_owners).
__device__ __forceinline__ uint32_t sp_pack(uint32_t f, uint32_t used, bool fast) {
    return f | (fast ? 8u : 0u) | (used << 4);
}
__device__ __forceinline__ uint32_t sp_used(uint32_t pc) { return (pc >> 4) & 0xfffu; }

// Edges whose vertex an earlier cell of the same x can make, in slot order:
// 0, 3, 4, 7, 8, 9, 11.
__host__ __device__ constexpr int sp_slot_edge(int s) {
    return s == 0 ? 0 : s == 1 ? 3 : s == 2 ? 4 : s == 3 ? 7 : s == 4 ? 8 : s == 5 ? 9 : 11;
}
constexpr unsigned long long sp_slot_table() {
    unsigned long long t = 0;
    for (int e = 0; e < 12; ++e) {
        int s = 7;
        for (int k = 0; k < 7; ++k)
            if (sp_slot_edge(k) == e) s = k;
        t |= (unsigned long long)s << (3 * e);
    }
    return t;
}
constexpr unsigned long long SP_SLOT = sp_slot_table();
__device__ __forceinline__ int sp_slot(int e) { return int((SP_SLOT >> (3 * e)) & 7ull); }

// The owner's edge for slot s and owner code k (1..3), a nibble of
// SP_SRC_{LO,HI} at 3 s + k - 1: e0 <- y e2; e3 <- z e1; e4 <- y e6;
// e7 <- z e5; e8 <- z e9, y e11, (y - 1, z - 1) e10; e9 <- y e10,
// (y - 1, z + 1) e11; e11 <- z e10 (the same lattice edge, corners in the
// same order).
constexpr int SP_SRC[21] = {0, 2, 0, 1, 0, 0, 0, 6, 0, 5, 0, 0, 9, 11, 10, 0, 10, 11, 10, 0, 0};
constexpr unsigned long long sp_src_table(int lo) {
    unsigned long long t = 0;
    for (int i = 0; i < 16; ++i)
        if (lo + i < 21) t |= (unsigned long long)SP_SRC[lo + i] << (4 * i);
    return t;
}
constexpr unsigned long long SP_SRC_LO = sp_src_table(0), SP_SRC_HI = sp_src_table(16);
__device__ __forceinline__ int sp_src_edge(int s, uint32_t k) {
    const int i = 3 * s + int(k) - 1;
    return int(((i < 16 ? SP_SRC_LO >> (4 * i) : SP_SRC_HI >> (4 * (i - 16)))) & 15ull);
}

// Edges whose entry is another cell's.
__device__ __forceinline__ uint32_t sp_reused(uint32_t pc) {
    uint32_t m = 0;
#pragma unroll
    for (int s = 0; s < 7; ++s) m |= ((pc >> (16 + 2 * s)) & 3u) ? (1u << sp_slot_edge(s)) : 0u;
    return m;
}
__device__ __forceinline__ uint32_t sp_own(uint32_t pc) { return sp_used(pc) & ~sp_reused(pc); }

__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }

__device__ __forceinline__ void load8(const float* vals, long long c, float* v) {
    const float4* p = reinterpret_cast<const float4*>(vals + 8 * c);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Owner codes of crossed cell c (list position j, id cid[j]) that keeps every
// triangle.  A lattice edge of the cell's x is shared with the cells at
// (y - 1 .. y, z - 1 .. z) around it; those of them in this chunk, earlier in
// the list, keeping every triangle and with the edge's two corner values the
// same bits as this cell's compute the same vertex (same operands, same corner
// positions).  Sameness is an equivalence, so the first such cell in the list
// makes the entry itself and every later one takes it: no chains.  The weld
// would merge the copies anyway; the emit points the triangles at the first.
__device__ __forceinline__ uint32_t sp_owners(const SpGrid& g, const float* vals, const uint16_t* list,
                                              const uint16_t* summ, const uint32_t* cid, long long c0, uint32_t j,
                                              uint32_t used, int& jy_out) {
    const uint32_t nzc = uint32_t(g.nz - 1);
    const uint32_t id = cid[j];
    const uint32_t z = id % nzc, y = (id / nzc) % uint32_t(g.ny - 1);
    int jz = -1, jy = -1, jyl = -1, jyh = -1;  // z-, y-, (y-1, z-1)-, (y-1, z+1)-neighbours
    if (z > 0 && j > 0 && cid[j - 1] == id - 1u && (summ[j - 1] & 8u)) jz = int(j) - 1;
    if (y > 0) {
        const uint32_t idy = id - nzc;
        uint32_t lo = 0, hi = j;  // first position with cid >= idy
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cid[mid] < idy) lo = mid + 1;
            else hi = mid;
        }
        // the diagonal cells are looked for whether the y-neighbour is listed or
        // not, as the cells that own through them look for them
        const bool hasy = lo < j && cid[lo] == idy;
        jy_out = int(lo) | (hasy ? 0x8000 : 0);
        if (hasy && (summ[lo] & 8u)) jy = int(lo);
        if (z > 0 && lo > 0 && cid[lo - 1] == idy - 1u && (summ[lo - 1] & 8u)) jyl = int(lo) - 1;
        const uint32_t ph = hasy ? lo + 1 : lo;
        if (z + 1 < nzc && ph < j && cid[ph] == idy + 1u && (summ[ph] & 8u)) jyh = int(ph);
    }
    if (jz < 0 && jy < 0 && jyl < 0 && jyh < 0) return 0u;
    float d[8], vz[8], vy[8], vl[8], vh[8];
    load8(vals, c0 + list[j], d);
    if (jz >= 0) load8(vals, c0 + list[jz], vz);
    if (jy >= 0) load8(vals, c0 + list[jy], vy);
    if (jyl >= 0) load8(vals, c0 + list[jyl], vl);
    if (jyh >= 0) load8(vals, c0 + list[jyh], vh);
    // the neighbour's corner k' holds this cell's corner k: z (k | 1), y (k | 2)
    const bool z0 = jz >= 0 && same_bits(d[0], vz[1]), z2 = jz >= 0 && same_bits(d[2], vz[3]);
    const bool z4 = jz >= 0 && same_bits(d[4], vz[5]), z6 = jz >= 0 && same_bits(d[6], vz[7]);
    const bool y0 = jy >= 0 && same_bits(d[0], vy[2]), y1 = jy >= 0 && same_bits(d[1], vy[3]);
    const bool y4 = jy >= 0 && same_bits(d[4], vy[6]), y5 = jy >= 0 && same_bits(d[5], vy[7]);
    uint32_t k = 0;
    if ((used & (1u << 0)) && y0 && y1) k |= 2u << 0;     // e0 (0, 1) <- y e2
    if ((used & (1u << 3)) && z0 && z2) k |= 1u << 2;     // e3 (0, 2) <- z e1
    if ((used & (1u << 4)) && y4 && y5) k |= 2u << 4;     // e4 (4, 5) <- y e6
    if ((used & (1u << 7)) && z4 && z6) k |= 1u << 6;     // e7 (4, 6) <- z e5
    if (used & (1u << 8)) {                               // e8 (0, 4), owners in list order
        if (jyl >= 0 && same_bits(d[0], vl[3]) && same_bits(d[4], vl[7])) k |= 3u << 8;
        else if (y0 && y4) k |= 2u << 8;
        else if (z0 && z4) k |= 1u << 8;
    }
    if (used & (1u << 9)) {                               // e9 (1, 5)
        if (y1 && y5) k |= 2u << 10;
        else if (jyh >= 0 && same_bits(d[1], vh[2]) && same_bits(d[5], vh[6])) k |= 3u << 10;
    }
    if ((used & (1u << 11)) && z2 && z6) k |= 1u << 12;   // e11 (2, 6) <- z e10
    return k;
}

// Per CTA: its crossed cells in cell order and, for each, sp_pack of its
// summary with the owner codes, into the chunk's slots of clist / ccnt / cjy
// (SP2_CHUNK each: cjy where id - (nz - 1) sorts in the list, bit 15 set when
// that cell is listed; the count in clen);
// the chunk's faces and vertex-list entries -> blk[2 b], blk[2 b + 1].  The
// emit then reads only the crossed cells.
__global__ void __launch_bounds__(SP2_THREADS) sp_mc_count2(SpGrid g, const int* __restrict__ ids,
                                                            const float* __restrict__ vals, long long n,
                                                            unsigned long long* blk, uint16_t* __restrict__ clist,
                                                            uint32_t* __restrict__ ccnt, uint16_t* __restrict__ cjy,
                                                            uint32_t* __restrict__ clen) {
    __shared__ uint16_t list[SP2_CHUNK];
    __shared__ uint16_t summ[SP2_CHUNK];  // sp_pack of each listed cell (16 bits)
    __shared__ uint32_t cid[SP2_CHUNK];   // their ids
    __shared__ uint32_t wcnt[SP2_ROUNDS][SP2_THREADS / 32];
    const long long c0 = (long long)blockIdx.x * SP2_CHUNK;
    const uint32_t nl = sp_crossed(g, vals, n, c0, list, wcnt);
    uint16_t* gl = clist + (size_t)blockIdx.x * SP2_CHUNK;
    uint32_t* gc = ccnt + (size_t)blockIdx.x * SP2_CHUNK;
    uint16_t* gy = cjy + (size_t)blockIdx.x * SP2_CHUNK;
    for (uint32_t j = threadIdx.x; j < nl; j += SP2_THREADS) {
        const long long c = c0 + list[j];
        Cell8 cc;
        const uint32_t cs = sp_case(g, vals, c, cc);
        float ev[12][3];
        uint32_t used;
        bool fast;
        const uint32_t f = sp_cell_summary(g, ids, c, cc, cs, ev, used, fast);
        summ[j] = uint16_t(sp_pack(f, used, fast));
        cid[j] = uint32_t(__ldg(ids + c));
    }
    __syncthreads();
    uint32_t nf = 0, nv = 0;
    for (uint32_t j = threadIdx.x; j < nl; j += SP2_THREADS) {
        uint32_t pc = summ[j];
        int jy = 0;
        if (pc & 8u) pc |= sp_owners(g, vals, list, summ, cid, c0, j, sp_used(pc), jy) << 16;
        gl[j] = list[j];
        gc[j] = pc;
        gy[j] = uint16_t(jy);
        nf += pc & 7u;
        nv += __popc(sp_own(pc));
    }
    sp_sum2(nf, nv, wcnt);
    if (threadIdx.x == 0) {
        blk[2 * blockIdx.x] = nf;
        blk[2 * blockIdx.x + 1] = nv;
        clen[blockIdx.x] = nl;
    }
}

// Output staging of one emit CTA: vertex-list entries and triangles up to
// these counts go through shared memory and leave in coalesced stores; a CTA
// with more (a dense patch of surface) writes the rest directly.
constexpr int SP2_STAGE_V = 2048;
constexpr int SP2_STAGE_F = 1024;

struct SpStage {
    float* v;                  // [SP2_STAGE_V * 3]
    int32_t* f;                // [SP2_STAGE_F * 3]
    float* gv;                 // the CTA's part of the vertex list
    int32_t* gf;               // the CTA's part of the triangles
    unsigned long long vbase;  // the CTA's first vertex-list entry
};

__device__ __forceinline__ void stage_vertex(const SpStage& s, uint32_t k, float x, float y, float z) {
    float* o = k < uint32_t(SP2_STAGE_V) ? s.v + 3 * k : s.gv + 3 * (size_t)k;
    o[0] = x; o[1] = y; o[2] = z;
}

// Staged triangles hold the CTA's own entry numbers (the copy-out adds the
// base); direct ones hold vertex-list indices.
__device__ __forceinline__ void stage_face(const SpStage& s, uint32_t k, uint32_t a, uint32_t b, uint32_t c) {
    if (k < uint32_t(SP2_STAGE_F)) {
        int32_t* o = s.f + 3 * k;
        o[0] = int32_t(a); o[1] = int32_t(b); o[2] = int32_t(c);
    } else {
        int32_t* o = s.gf + 3 * (size_t)k;
        o[0] = int32_t(s.vbase + a); o[1] = int32_t(s.vbase + b); o[2] = int32_t(s.vbase + c);
    }
}

// A cell with a vertex near a corner: its triangles are kept by position
// (as mc_cell does), so every crossed edge's position is needed.  Its
// position array is indexed by the triangle table and lives in local memory;
// the common path (no vertex near a corner) never touches it.
__device__ __forceinline__ void sp_emit_near(const SpGrid& g, const Cell8& cc, uint32_t cs, uint32_t used,
                                          unsigned long long pk, const SpStage& s, uint32_t lv, uint32_t lf) {
    float ev[12][3];
    const uint32_t est = ISO_EDGE_STATUS[cs];
#pragma unroll
    for (int e = 0; e < 12; ++e)
        if ((est >> e) & 1u) edge_point(cc, e, g.level, ev[e]);
#pragma unroll
    for (int q = 0; q < 12; ++q)
        if ((used >> q) & 1u) stage_vertex(s, lv + __popc(used & ((1u << q) - 1u)), ev[q][0], ev[q][1], ev[q][2]);
    const int ntc = int(pk >> 60);
    for (int t = 0; t < ntc; ++t, pk >>= 12) {
        const int a = int(pk & 15u), b = int((pk >> 4) & 15u), d = int((pk >> 8) & 15u);
        if (eq3(ev[a], ev[b]) || eq3(ev[a], ev[d]) || eq3(ev[b], ev[d])) continue;
        stage_face(s, lf++, lv + __popc(used & ((1u << a) - 1u)), lv + __popc(used & ((1u << b) - 1u)),
                   lv + __popc(used & ((1u << d) - 1u)));
    }
}

// Per CTA: its crossed cells in cell order (from the count pass), 256 per
// round; a block scan of each round's (faces, vertices) gives every cell its
// offsets in list order.  A cell writes its used vertices in edge order and
// its kept triangles as indices into the vertex list.  dn (device): nothing
// is written when dn[0] == 0 (over capacity).
__global__ void __launch_bounds__(SP2_THREADS) sp_mc_emit2(SpGrid g, const int* __restrict__ ids,
                                                           const float* __restrict__ vals, long long n,
                                                           const unsigned long long* __restrict__ blk,
                                                           const uint16_t* __restrict__ clist,
                                                           const uint32_t* __restrict__ ccnt,
                                                           const uint16_t* __restrict__ cjy,
                                                           const uint32_t* __restrict__ clen,
                                                           float* __restrict__ vlist, int32_t* __restrict__ tri,
                                                           const long long* __restrict__ dn) {
    __shared__ unsigned long long tpk[256];  // packed triangle lists of the cases
    __shared__ float sv[SP2_STAGE_V * 3];
    __shared__ int32_t sf[SP2_STAGE_F * 3];
    __shared__ uint32_t wsum[2][SP2_THREADS / 32];
    __shared__ uint16_t slv[SP2_CHUNK];  // each listed cell's first own entry (CTA-local)
    if (dn[0] == 0) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 256; i += SP2_THREADS) tpk[i] = ISO_TRI_PACKED[g.method * 256 + i];
    const long long c0 = (long long)blockIdx.x * SP2_CHUNK;
    const uint32_t nl = clen[blockIdx.x];
    const uint16_t* gl = clist + (size_t)blockIdx.x * SP2_CHUNK;
    const uint32_t* gc = ccnt + (size_t)blockIdx.x * SP2_CHUNK;
    const uint16_t* gy = cjy + (size_t)blockIdx.x * SP2_CHUNK;
    SpStage s;
    s.v = sv;
    s.f = sf;
    s.vbase = blk[2 * blockIdx.x + 1];
    s.gv = vlist + 3 * s.vbase;
    s.gf = tri + 3 * blk[2 * blockIdx.x];
    uint32_t accf = 0, accv = 0;  // faces and vertices of the rounds before
    for (uint32_t r0 = 0; r0 < nl; r0 += SP2_THREADS) {
        const uint32_t j = r0 + threadIdx.x;
        const bool ok = j < nl;
        const uint32_t pc = ok ? gc[j] : 0u;
        const uint32_t cl = ok ? gl[j] : 0u;
        const uint32_t used = sp_used(pc), own = sp_own(pc);
        const uint32_t mine = (pc & 7u) | (uint32_t(__popc(own)) << 16);  // faces | own vertices << 16
        uint32_t inc = mine;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(~0u, inc, d);
            if (lane >= d) inc += o;
        }
        const int buf = (r0 / SP2_THREADS) & 1;  // alternate buffers between rounds
        if (lane == 31) wsum[buf][warp] = inc;
        __syncthreads();  // also orders tpk's fill before its first use
        uint32_t before = 0, all = 0;
#pragma unroll
        for (int k = 0; k < SP2_THREADS / 32; ++k) {
            const uint32_t w = wsum[buf][k];
            before += k < warp ? w : 0u;
            all += w;
        }
        const uint32_t ex = before + inc - mine;
        const uint32_t lv = accv + (ex >> 16), lf = accf + (ex & 0xffffu);
        if (ok) slv[j] = uint16_t(lv);
        __syncthreads();  // first entries of this round's cells, for the cells that take them
        if (ok) {
            const long long c = c0 + cl;
            Cell8 cc;
            const uint32_t cs = sp_case(g, vals, c, cc);
            int x, y, z;
            cell_xyz(g, uint32_t(ids[c]), x, y, z);
            set_coords(g, x, y, z, cc);
            const unsigned long long pk = tpk[cs];
            if (pc & 8u) {  // every triangle kept, every crossed edge used
#pragma unroll
                for (int q = 0; q < 12; ++q)
                    if ((own >> q) & 1u) {
                        float p[3];
                        edge_point(cc, q, g.level, p);
                        stage_vertex(s, lv + __popc(own & ((1u << q) - 1u)), p[0], p[1], p[2]);
                    }
                // entry of each edge: the cell's own, or its owner's (an earlier
                // listed cell: first entry from slv, rank among the owner's own edges)
                const uint32_t codes = pc >> 16;
                const uint32_t lo = codes & 0x1555u, hi = (codes >> 1) & 0x1555u;
                uint32_t oz = 0, lz = 0, oy = 0, ly = 0, ol = 0, ll = 0, oh = 0, lh = 0;
                if (lo & ~hi) { oz = sp_own(gc[j - 1]); lz = slv[j - 1]; }
                if (codes) {
                    // where id - (nz - 1) sorts in the list, and whether that cell is listed
                    const uint32_t py = gy[j] & 0x7fffu, hasy = gy[j] >> 15;
                    if (hi & ~lo) { oy = sp_own(gc[py]); ly = slv[py]; }
                    if (((codes >> 8) & 3u) == 3u) { ol = sp_own(gc[py - 1]); ll = slv[py - 1]; }
                    if (((codes >> 10) & 3u) == 3u) {
                        const uint32_t ph = py + hasy;
                        oh = sp_own(gc[ph]);
                        lh = slv[ph];
                    }
                }
                unsigned long long ent[3] = {0ull, 0ull, 0ull};  // 16 bits per edge
#pragma unroll
                for (int q = 0; q < 12; ++q) {
                    const int sl = sp_slot(q);
                    const uint32_t k = sl < 7 ? (codes >> (2 * sl)) & 3u : 0u;
                    uint32_t e;
                    if (k == 0u) {
                        e = lv + __popc(own & ((1u << q) - 1u));
                    } else {
                        const uint32_t se = uint32_t(sp_src_edge(sl, k));
                        const uint32_t ob = k == 1u ? oz : (k == 2u ? oy : (q == 8 ? ol : oh));
                        const uint32_t lb = k == 1u ? lz : (k == 2u ? ly : (q == 8 ? ll : lh));
                        e = lb + __popc(ob & ((1u << se) - 1u));
                    }
                    ent[q >> 2] |= (unsigned long long)(e & 0xffffu) << (16 * (q & 3));
                }
                unsigned long long t = pk;
                const int ntc = int(pk >> 60);
                for (int k = 0; k < ntc; ++k, t >>= 12) {
                    uint32_t v3[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        const uint32_t e = uint32_t((t >> (4 * r)) & 15u);
                        const unsigned long long w = e < 4u ? ent[0] : (e < 8u ? ent[1] : ent[2]);
                        v3[r] = uint32_t((w >> (16 * (e & 3u))) & 0xffffu);
                    }
                    stage_face(s, lf + k, v3[0], v3[1], v3[2]);
                }
            } else {
                sp_emit_near(g, cc, cs, used, pk, s, lv, lf);
            }
        }
        accf += all & 0xffffu;
        accv += all >> 16;
    }
    __syncthreads();
    const uint32_t nv = 3 * min(accv, uint32_t(SP2_STAGE_V)), nf = 3 * min(accf, uint32_t(SP2_STAGE_F));
    for (uint32_t i = threadIdx.x; i < nv; i += SP2_THREADS) s.gv[i] = sv[i];
    for (uint32_t i = threadIdx.x; i < nf; i += SP2_THREADS) s.gf[i] = int32_t(s.vbase + sf[i]);
}

// --- intersections -----------------------------------------------------------

// Normal at crossing point p (src/its.cu:186-268).
__device__ __forceinline__ void cell_normal(const Cell8& cc, const float* p, float* n) {
    iso::stencil_normal(cc.v, cc.p[0], cc.p[7], p, n, cc.fma);
}

__global__ void __launch_bounds__(SP_BLOCK) sp_its_count(SpGrid g, const float* __restrict__ vals,
                                                         long long n, unsigned long long* blk) {
    __shared__ uint32_t sm[33];
    __shared__ uint32_t sk[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t na = 0, nk = 0;
    if (c < n) {
        uint32_t cs = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) cs |= (iso::below(vals[8 * c + k], g.level) ? 1u : 0u) << k;
        nk = __popc(uint32_t(ISO_EDGE_STATUS[cs]));
        na = nk ? 1u : 0u;
    }
    uint32_t e, ta, tk;
    block_scan1(na, e, ta, sm);
    block_scan1(nk, e, tk, sk);
    if (threadIdx.x == 0) { blk[2 * blockIdx.x] = ta; blk[2 * blockIdx.x + 1] = tk; }
}

__global__ void __launch_bounds__(SP_BLOCK) sp_its_emit(SpGrid g, const int* __restrict__ ids,
                                                        const float* __restrict__ vals, long long n,
                                                        const unsigned long long* __restrict__ blk,
                                                        float* points, float* normals, int* act_sparse,
                                                        int* act_uniform, int* offsets, uint32_t* rank,
                                                        long long A, long long K) {
    __shared__ uint32_t sm[33];
    __shared__ uint32_t sk[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t na = 0, nk = 0, est = 0;
    if (c < n) {
        uint32_t cs = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) cs |= (iso::below(vals[8 * c + k], g.level) ? 1u : 0u) << k;
        est = ISO_EDGE_STATUS[cs];
        nk = __popc(est);
        na = nk ? 1u : 0u;
    }
    uint32_t ea, ek, ta, tk;
    block_scan1(na, ea, ta, sm);
    block_scan1(nk, ek, tk, sk);
    if (c >= n) return;
    const unsigned long long a = blk[2 * blockIdx.x] + ea;
    rank[c] = na ? uint32_t(a) : 0xffffffffu;
    if (!na) return;
    unsigned long long k = blk[2 * blockIdx.x + 1] + ek;
    Cell8 cc;
    int x, y, z;
    load_cell(g, ids, vals, c, cc, x, y, z);
    act_sparse[a] = int(c);
    act_uniform[a] = ids[c];
    offsets[a] = int(k);
    for (uint32_t em = est; em; em &= em - 1) {  // this lane's crossed edges, ascending
        const int e = __ffs(em) - 1;
        float p[3];
        edge_point(cc, e, g.level, p);
        points[3 * k] = p[0]; points[3 * k + 1] = p[1]; points[3 * k + 2] = p[2];
        if (normals) {
            float nn[3];
            cell_normal(cc, p, nn);
            normals[3 * k] = nn[0]; normals[3 * k + 1] = nn[1]; normals[3 * k + 2] = nn[2];
        }
        ++k;
    }
    if (a + 1 == (unsigned long long)A) offsets[A] = int(K);
}

// Normals of an existing sparse intersection.
__global__ void sp_normals(SpGrid g, const int* __restrict__ ids, const float* __restrict__ vals,
                           const int* __restrict__ act_sparse, const int* __restrict__ offsets, long long A,
                           const float* __restrict__ points, float* normals) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    Cell8 cc;
    int x, y, z;
    load_cell(g, ids, vals, act_sparse[a], cc, x, y, z);
    for (int k = offsets[a]; k < offsets[a + 1]; ++k) {
        const float p[3] = {points[3 * k], points[3 * k + 1], points[3 * k + 2]};
        float nn[3];
        cell_normal(cc, p, nn);
        normals[3 * k] = nn[0]; normals[3 * k + 1] = nn[1]; normals[3 * k + 2] = nn[2];
    }
}

// --- quads ---------------------------------------------------------------------

__device__ __forceinline__ long long find_cell(const int* ids, long long n, uint32_t id) {
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (uint32_t(ids[mid]) < id) lo = mid + 1; else hi = mid;
    }
    return (lo < n && uint32_t(ids[lo]) == id) ? lo : -1;
}

// Edge (corner a -> corner b of cell s) crossed according to sparse cell s.
__device__ __forceinline__ int edge_sign(const float* vals, long long s, int a, int b, float level) {
    const bool ba = iso::below(vals[8 * s + a], level), bb = iso::below(vals[8 * s + b], level);
    return ba == bb ? -1 : (ba ? 1 : 0);  // -1 not crossed; else is_out = low endpoint below
}

// For cell c's edge along `ax` at its lowest corner: the quad's 4 sparse cells
// and its orientation; false when it has no quad.
__device__ bool cell_quad(const SpGrid& g, const int* ids, const float* vals, long long n, long long c, int ax,
                          long long* q, bool& out) {
    int x, y, z;
    cell_xyz(g, uint32_t(ids[c]), x, y, z);
    // edge_neighbors_table (src/shared_luts.cu:78-81): cells p - o_i
    const int o[3][4][3] = {{{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}},
                            {{0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 0, 0}},
                            {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}}};
    // the edge, as corners of a neighbour cell whose offset is (dx, dy, dz):
    // its low corner is at (dx, dy, dz) relative to that cell
    const int step = ax == 0 ? 4 : (ax == 1 ? 2 : 1);
    int crossed = -1;
    long long first = -1;
    for (int i = 0; i < 4; ++i) {
        const int cx = x - o[ax][i][0], cy = y - o[ax][i][1], cz = z - o[ax][i][2];
        if (cx < 0 || cy < 0 || cz < 0 || cx > g.nx - 2 || cy > g.ny - 2 || cz > g.nz - 2) return false;
        const uint32_t id = (uint32_t(cx) * uint32_t(g.ny - 1) + uint32_t(cy)) * uint32_t(g.nz - 1) + uint32_t(cz);
        q[i] = find_cell(ids, n, id);
        if (q[i] < 0) return false;
    }
    // crossing status: isoext keeps an edge if any cell reports it crossed; its
    // orientation comes from the first such cell in sparse order
    for (int i = 0; i < 4; ++i) {
        const int ca = 4 * o[ax][i][0] + 2 * o[ax][i][1] + o[ax][i][2];
        const int s = edge_sign(vals, q[i], ca, ca + step, g.level);
        if (s >= 0 && (first < 0 || q[i] < first)) {
            first = q[i];
            crossed = s;
        }
    }
    if (crossed < 0) return false;
    out = crossed == 1;
    return true;
}

__global__ void __launch_bounds__(SP_BLOCK) sp_quad_count(SpGrid g, const int* __restrict__ ids,
                                                          const float* __restrict__ vals, long long n,
                                                          const uint32_t* __restrict__ rank,
                                                          unsigned long long* blk) {
    __shared__ uint32_t sm[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t nq = 0;
    if (c < n) {
        for (int ax = 2; ax >= 0; --ax) {
            long long q[4];
            bool out;
            if (!cell_quad(g, ids, vals, n, c, ax, q, out)) continue;
            bool ok = true;
            for (int i = 0; i < 4; ++i) ok &= rank[q[i]] != 0xffffffffu;
            nq += ok;
        }
    }
    uint32_t e, t;
    block_scan1(nq, e, t, sm);
    if (threadIdx.x == 0) { blk[2 * blockIdx.x] = t; blk[2 * blockIdx.x + 1] = 0; }
}

// |a - b| (norm(v0 - v2) of src/dc.cu:139), in the grid's arithmetic reading.
__device__ __forceinline__ float dist3(const float* a, const float* b, bool fma) {
    const float dx = __fsub_rn(a[0], b[0]), dy = __fsub_rn(a[1], b[1]), dz = __fsub_rn(a[2], b[2]);
    return iso::norm3f(dx, dy, dz, fma);
}

__global__ void __launch_bounds__(SP_BLOCK) sp_quad_emit(SpGrid g, const int* __restrict__ ids,
                                                         const float* __restrict__ vals, long long n,
                                                         const uint32_t* __restrict__ rank,
                                                         const unsigned long long* __restrict__ blk,
                                                         const float* __restrict__ dual, int* tri) {
    __shared__ uint32_t sm[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t nq = 0;
    long long qs[3][4];
    bool outs[3], oks[3] = {false, false, false};
    if (c < n) {
        for (int ax = 2; ax >= 0; --ax) {
            if (!cell_quad(g, ids, vals, n, c, ax, qs[ax], outs[ax])) continue;
            bool ok = true;
            for (int i = 0; i < 4; ++i) ok &= rank[qs[ax][i]] != 0xffffffffu;
            oks[ax] = ok;
            nq += ok;
        }
    }
    uint32_t e, t;
    block_scan1(nq, e, t, sm);
    if (!nq) return;
    unsigned long long qo = blk[2 * blockIdx.x] + e;
    for (int ax = 2; ax >= 0; --ax) {
        if (!oks[ax]) continue;
        int32_t qi[4];
        for (int i = 0; i < 4; ++i) qi[i] = int32_t(rank[qs[ax][i]]);
        if (!outs[ax]) {
            const int32_t t0 = qi[0], t1 = qi[1];
            qi[0] = qi[3]; qi[1] = qi[2]; qi[2] = t1; qi[3] = t0;
        }
        float v[4][3];
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) v[i][k] = dual[3 * (long long)qi[i] + k];
        int* o6 = tri + 6 * qo;
        if (dist3(v[0], v[2], g.fma) > dist3(v[1], v[3], g.fma)) {
            o6[0] = qi[1]; o6[1] = qi[3]; o6[2] = qi[0]; o6[3] = qi[3]; o6[4] = qi[1]; o6[5] = qi[2];
        } else {
            o6[0] = qi[2]; o6[1] = qi[0]; o6[2] = qi[1]; o6[3] = qi[0]; o6[4] = qi[2]; o6[5] = qi[3];
        }
        ++qo;
    }
}

// --- population helpers ------------------------------------------------------

// Corner positions [M, 8, 3] of cells given by linear id.
__global__ void sp_points(SpGrid g, const int* __restrict__ ids, long long m, float* out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m * 8) return;
    const long long c = i >> 3;
    const int k = int(i & 7);
    int x, y, z;
    cell_xyz(g, uint32_t(ids[c]), x, y, z);
    out[3 * i] = iso::grid_coord(x + (k >> 2), g.nx, g.amin[0], g.asize[0], g.fma);
    out[3 * i + 1] = iso::grid_coord(y + ((k >> 1) & 1), g.ny, g.amin[1], g.asize[1], g.fma);
    out[3 * i + 2] = iso::grid_coord(z + (k & 1), g.nz, g.amin[2], g.asize[2], g.fma);
}

// Keep the ids whose 8 values straddle the level (src/grid/sparse.cu:150-179),
// in input order.
__global__ void __launch_bounds__(SP_BLOCK) sp_filter_count(const float* __restrict__ vals, long long m,
                                                            float level, unsigned long long* blk) {
    __shared__ uint32_t sm[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t keep = 0;
    if (c < m) {
        uint32_t cs = 0;
        for (int k = 0; k < 8; ++k) cs |= (iso::below(vals[8 * c + k], level) ? 1u : 0u) << k;
        keep = (cs != 0 && cs != 255);
    }
    uint32_t e, t;
    block_scan1(keep, e, t, sm);
    if (threadIdx.x == 0) { blk[2 * blockIdx.x] = t; blk[2 * blockIdx.x + 1] = 0; }
}

__global__ void __launch_bounds__(SP_BLOCK) sp_filter_write(const int* __restrict__ ids,
                                                            const float* __restrict__ vals, long long m,
                                                            float level,
                                                            const unsigned long long* __restrict__ blk,
                                                            int* out) {
    __shared__ uint32_t sm[33];
    const long long c = (long long)blockIdx.x * SP_BLOCK + threadIdx.x;
    uint32_t keep = 0;
    if (c < m) {
        uint32_t cs = 0;
        for (int k = 0; k < 8; ++k) cs |= (iso::below(vals[8 * c + k], level) ? 1u : 0u) << k;
        keep = (cs != 0 && cs != 255);
    }
    uint32_t e, t;
    block_scan1(keep, e, t, sm);
    if (keep) out[blk[2 * blockIdx.x] + e] = ids[c];
}

SpGrid mk(int nx, int ny, int nz, const float* amin, const float* amax, float level, int method) {
    SpGrid g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    for (int k = 0; k < 3; ++k) { g.amin[k] = amin[k]; g.asize[k] = amax[k] - amin[k]; }
    g.level = level;
    g.method = method;
    g.tau = snap_tau_box(nx, ny, nz, g.amin, g.asize);
    g.fma = iso::arith_fma();
    return g;
}
unsigned nb(long long n, int b) { return unsigned(std::max<long long>(1, (n + b - 1) / b)); }

}  // namespace

// dc_block_scan lives in dc_dense.cu
void iso_block_scan_launch(unsigned long long* blk, long long nblk, long long* totals, cudaStream_t st);
// dc_dense.cu: exact-position weld with device-side sizes
size_t weld_dev_workspace(long long capA, long long capU);
void weld_dev_launch(const float* pts, long long capA, long long capU, const int32_t* tri, long long capT,
                     const long long* eff,
                     void* ws, float* vout, int32_t* fout, long long* vtot, int* status, cudaStream_t st,
                     uint32_t* vsrc);

namespace {

// The list's and the faces' sizes against the capacities: eff = (vertex-list
// entries, 0, 3 F, vertex capacity) for the weld, all 0 when they do not fit.
__global__ void sp_mc_sizes2(const long long* __restrict__ tot, long long capF, long long capV, long long* eff,
                             long long* counts, int* status) {
    const long long F = tot[0], L = tot[1];
    const bool ok = F <= capF && L <= 3 * capF && 3 * F < 0x7fffffffll;
    if (!ok) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
    eff[0] = ok ? L : 0;
    eff[1] = 0;
    eff[2] = ok ? 3 * F : 0;
    eff[3] = capV;
    counts[1] = ok ? F : 0;
    counts[2] = F;
}

__global__ void sp_mc_finish(const long long* __restrict__ vtot, long long capV, long long* counts, int* status) {
    const long long V = vtot[0];
    counts[0] = V;
    if (V > capV) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
}

struct SpMcWs {
    void* blk;
    long long* tot;  // [0..1] F, vertex-list entries  [4..7] eff  [8..9] V, 0
    float* soup;     // the vertex list (at most 3 F entries)
    int32_t* tri;    // the triangles' indices into it [3 F]
    uint16_t* clist;  // per chunk: crossed cells (SP2_CHUNK slots each)
    uint32_t* ccnt;   // per chunk: their summaries (sp_pack)
    uint16_t* cjy;    // per chunk: where their y-neighbours sort in the list (bit 15: listed)
    uint32_t* clen;          // per chunk: crossed cells
    void* weld;
    size_t total;
};

SpMcWs sp_mc_carve(void* ws, long long n, long long capV, long long capF) {
    SpMcWs w{};
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = ws ? b + o : nullptr;
        o = (o + std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        return p;
    };
    w.blk = take(size_t((n + SP2_CHUNK - 1) / SP2_CHUNK + 1) * 16);
    w.tot = reinterpret_cast<long long*>(take(16 * 8));
    w.soup = reinterpret_cast<float*>(take(size_t(3 * capF) * 12));
    w.tri = reinterpret_cast<int32_t*>(take(size_t(3 * capF) * 4));
    const size_t chunks = size_t((n + SP2_CHUNK - 1) / SP2_CHUNK);
    w.clist = reinterpret_cast<uint16_t*>(take(chunks * SP2_CHUNK * 2));
    w.ccnt = reinterpret_cast<uint32_t*>(take(chunks * SP2_CHUNK * 4));
    w.cjy = reinterpret_cast<uint16_t*>(take(chunks * SP2_CHUNK * 2));
    w.clen = reinterpret_cast<uint32_t*>(take(chunks * 4));
    w.weld = take(weld_dev_workspace(3 * capF, capV));
    w.total = o + 256;
    return w;
}

}  // namespace

extern "C" {

// Block sums workspace: 16 bytes per 1024 entries.
size_t iso_sparse_blocks_size(long long n) { return size_t((n + SP_BLOCK - 1) / SP_BLOCK + 1) * 16 + 256; }

int iso_sparse_mc_count(const int* ids, const float* vals, long long n, int nx, int ny, int nz,
                        const float* amin, const float* amax, float level, int method, void* blk,
                        long long* counts, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n <= 0) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    if (method != 0 && method != 1) return iso::fail_code(ISO_ERR_ARG);
    SpGrid g = mk(nx, ny, nz, amin, amax, level, method);
    iso::ProfScope ps("sparse_mc", st, 2);
    sp_mc_count<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, ids, vals, n, (unsigned long long*)blk);
    iso_block_scan_launch((unsigned long long*)blk, nb(n, SP_BLOCK), counts, st);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_mc_emit(const int* ids, const float* vals, long long n, int nx, int ny, int nz,
                       const float* amin, const float* amax, float level, int method, const void* blk,
                       float* soup, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n <= 0) return 0;
    SpGrid g = mk(nx, ny, nz, amin, amax, level, method);
    iso::ProfScope ps("sparse_mc", st);
    sp_mc_emit<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, ids, vals, n, (const unsigned long long*)blk, soup, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_its_count(const float* vals, long long n, float level, void* blk, long long* counts,
                         void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n <= 0) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    SpGrid g{};
    g.level = level;
    iso::ProfScope ps("sparse_its", st, 2);
    sp_its_count<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, vals, n, (unsigned long long*)blk);
    iso_block_scan_launch((unsigned long long*)blk, nb(n, SP_BLOCK), counts, st);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

// Intersection arrays; act_sparse / act_uniform: sparse index / lattice id of
// each active cell; rank[n]: active index of each sparse cell (or -1).
int iso_sparse_its_emit(const int* ids, const float* vals, long long n, int nx, int ny, int nz,
                        const float* amin, const float* amax, float level, const void* blk, long long A,
                        long long K, float* points, float* normals, int* act_sparse, int* act_uniform,
                        int* offsets, int* rank, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A == 0 && offsets) cudaMemsetAsync(offsets, 0, 4, st);
    if (n <= 0) return 0;
    SpGrid g = mk(nx, ny, nz, amin, amax, level, 0);
    iso::ProfScope ps("sparse_its", st);
    sp_its_emit<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, ids, vals, n, (const unsigned long long*)blk, points,
                                                      normals, act_sparse, act_uniform, offsets,
                                                      reinterpret_cast<uint32_t*>(rank), A, K);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_normals(const int* ids, const float* vals, int nx, int ny, int nz, const float* amin,
                       const float* amax, const int* act_sparse, const int* offsets, long long A,
                       const float* points, float* normals, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A <= 0) return 0;
    SpGrid g = mk(nx, ny, nz, amin, amax, 0.0f, 0);
    iso::ProfScope ps("sparse_its", st);
    sp_normals<<<nb(A, 256), 256, 0, st>>>(g, ids, vals, act_sparse, offsets, A, points, normals);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_quads_count(const int* ids, const float* vals, long long n, int nx, int ny, int nz,
                           float level, const int* rank, void* blk, long long* counts, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n <= 0) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    const float z3[3] = {0, 0, 0}, o3[3] = {1, 1, 1};
    SpGrid g = mk(nx, ny, nz, z3, o3, level, 0);
    iso::ProfScope ps("sparse_quads", st, 2);
    sp_quad_count<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, ids, vals, n, reinterpret_cast<const uint32_t*>(rank),
                                                        (unsigned long long*)blk);
    iso_block_scan_launch((unsigned long long*)blk, nb(n, SP_BLOCK), counts, st);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_quads_emit(const int* ids, const float* vals, long long n, int nx, int ny, int nz, float level,
                          const int* rank, const void* blk, const float* dual, int* tri, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (n <= 0) return 0;
    const float z3[3] = {0, 0, 0}, o3[3] = {1, 1, 1};
    SpGrid g = mk(nx, ny, nz, z3, o3, level, 0);
    iso::ProfScope ps("sparse_quads", st);
    sp_quad_emit<<<nb(n, SP_BLOCK), SP_BLOCK, 0, st>>>(g, ids, vals, n, reinterpret_cast<const uint32_t*>(rank),
                                                       (const unsigned long long*)blk, dual, tri);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_points(const int* ids, long long m, int nx, int ny, int nz, const float* amin,
                      const float* amax, float* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (m <= 0) return 0;
    SpGrid g = mk(nx, ny, nz, amin, amax, 0.0f, 0);
    iso::ProfScope ps("sparse_populate", st);
    sp_points<<<nb(m * 8, 256), 256, 0, st>>>(g, ids, m, out);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_filter_count(const float* vals, long long m, float level, void* blk, long long* counts,
                            void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (m <= 0) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    iso::ProfScope ps("sparse_populate", st, 2);
    sp_filter_count<<<nb(m, SP_BLOCK), SP_BLOCK, 0, st>>>(vals, m, level, (unsigned long long*)blk);
    iso_block_scan_launch((unsigned long long*)blk, nb(m, SP_BLOCK), counts, st);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_sparse_filter_write(const int* ids, const float* vals, long long m, float level, const void* blk,
                            int* out, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (m <= 0) return 0;
    iso::ProfScope ps("sparse_populate", st);
    sp_filter_write<<<nb(m, SP_BLOCK), SP_BLOCK, 0, st>>>(ids, vals, m, level, (const unsigned long long*)blk, out);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

// Sparse marching cubes in one call with no host synchronisation: the triangle
// soup and its exact-position weld (isoext's sparse MC, src/grid/sparse.cu with
// src/mc/mc.cu:17-68).  counts (device int64[3]) <- (V, F, F needed); status 6
// when F > face_capacity or V > vertex_capacity, and a retry sizes from counts.
size_t iso_sparse_mc_workspace_size(long long n, long long vertex_capacity, long long face_capacity) {
    if (n < 0 || vertex_capacity < 0 || face_capacity < 0) return 0;
    return sp_mc_carve(nullptr, n, vertex_capacity, face_capacity).total;
}

int iso_sparse_mc(const int* ids, const float* vals, long long n, int nx, int ny, int nz, const float* amin,
                  const float* amax, float level, int method, float* vertices, long long vertex_capacity, int* faces,
                  long long face_capacity, void* workspace, size_t workspace_bytes, long long* counts, int* status,
                  void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!counts || !status || !amin || !amax || n < 0 || vertex_capacity < 0 || face_capacity < 0) return iso::fail_code(ISO_ERR_ARG);
    if (method != 0 && method != 1) return iso::fail_code(ISO_ERR_ARG);
    if (n == 0) return cudaMemsetAsync(counts, 0, 24, st) == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
    if (!ids || !vals || (vertex_capacity && !vertices) || (face_capacity && !faces)) return iso::fail_code(ISO_ERR_ARG);
    if (workspace_bytes < iso_sparse_mc_workspace_size(n, vertex_capacity, face_capacity)) return iso::fail_code(ISO_ERR_WORKSPACE);
    const SpMcWs w = sp_mc_carve(workspace, n, vertex_capacity, face_capacity);
    const SpGrid g = mk(nx, ny, nz, amin, amax, level, method);
    long long* eff = w.tot + 4;
    {
        iso::ProfScope ps("sparse_mc", st, 4);
        const unsigned chunks = nb(n, SP2_CHUNK);
        sp_mc_count2<<<chunks, SP2_THREADS, 0, st>>>(g, ids, vals, n, (unsigned long long*)w.blk, w.clist, w.ccnt,
                                                     w.cjy, w.clen);
        iso_block_scan_launch((unsigned long long*)w.blk, chunks, w.tot, st);
        sp_mc_sizes2<<<1, 1, 0, st>>>(w.tot, face_capacity, vertex_capacity, eff, counts, status);
        sp_mc_emit2<<<chunks, SP2_THREADS, 0, st>>>(g, ids, vals, n, (const unsigned long long*)w.blk, w.clist,
                                                    w.ccnt, w.cjy, w.clen, w.soup, w.tri, eff);
    }
    // the weld of the vertex list: its table holds vertex_capacity distinct
    // positions; more report an overflow with a vertex count that fits on the rerun
    weld_dev_launch(w.soup, 3 * face_capacity, std::max<long long>(vertex_capacity, 1), w.tri, 3 * face_capacity,
                    eff, w.weld, vertices, faces, w.tot + 8, status, st, nullptr);
    {
        iso::ProfScope ps("sparse_mc", st);
        sp_mc_finish<<<1, 1, 0, st>>>(w.tot + 8, vertex_capacity, counts, status);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

}  // extern "C"
