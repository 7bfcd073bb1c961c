// Dense-grid marching cubes on sm_103a.
//
// Four launches on one stream, nothing read back by the host:
//   1. mc_signs   streams the grid once (one warp per row, 16 coalesced
//                 128-byte loads in flight per warp) into a sign bitmap,
//                 1 bit per point.  This is the only pass over all values.
//   2. mc_count   one CTA per segment of 1024 point words, from the bitmap alone
//                 (16.8 MB at 512^3): crossed-edge masks along x, y and z, active
//                 cells (their triangle counts spread over the lanes of a warp);
//                 segment-local vertex offsets per word; words with vertices or
//                 faces are appended to a list (one atomic per warp).  Words
//                 wholly inside or outside take an early exit.
//   3. mc_scan    segment (V, F) sums to offsets: CTAs over chunks of 4096
//                 segments chained by decoupled look-back; totals and the
//                 capacity check.
//   4. mc_emit    warp-cooperative over the listed words: each lane takes one
//                 vertex (position at its slot; values are read only at crossed
//                 edges), then one active cell (faces at the word's face offset,
//                 vertex indices by rank).  Vertices that can share a position
//                 with another edge's (t within tau of 0 or 1) go through a small
//                 hash that counts exact coincidences.
//   The last emit CTA to finish does the fix-up when the emit kernel found
//   coinciding vertices: it merges them by exact position, drops faces that
//   became degenerate and compacts vertices and faces, keeping their order.
//
// Equivalence with the reference (src/mc/mc.cu:17-68): the reference emits the
// triangles of active cells in ascending cell id, drops triangles with two equal
// vertex positions (src/mc/nagae.cu:71), and welds vertices by exact position
// (src/utils.cu:32-59).  Positions here use the reference's operation order
// and its rounding, in either reading of its arithmetic (the fused one of its
// CUDA build or the unfused one of its host build, common.cuh), so they are
// bit-identical.  Two
// distinct crossed edges give equal positions only when both vertices land on
// the same grid point (on grids whose spacing is far above float resolution;
// the host layer handles the rest), and those are the snapped vertices the
// fix-up merges.  Every crossed edge of a cell appears in its triangles (both
// tables), so without snaps the vertex set is exactly the crossed edges.
// Vertices come in edge order (the reference sorts them by position; the mesh
// is the same after relabelling).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "lookback.cuh"
#include "mc_dense.cuh"
#include "profile.cuh"

namespace {

// ---------------------------------------------------------------------------
// Geometry shared by the kernels.

// Unsigned 32-bit division by a divisor fixed for a launch, by multiply and
// shift (Granlund and Montgomery, "Division by invariant integers using
// multiplication", 1994): for 1 <= d < 2^31, l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (t + ((n - t) >> 1)) >> (l - 1) with
// t = umulhi(m, n); exact for every 32-bit n.
struct FastDiv {
    uint32_t d, m, l;
};

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f{d, 0u, 0u};
    while ((1ull << f.l) < d) ++f.l;
    if (d > 1) f.m = uint32_t(((1ull << 32) * ((1ull << f.l) - d)) / d + 1);
    return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    if (f.d == 1) return n;
    const uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> 1)) >> (f.l - 1);
}

struct McGrid {
    FastDiv dNW, dNY;  // division by NW and by ny
    int nx, ny, nz, NW;
    long long PW;     // point words nx * ny * NW
    float level;
    int method;
    const float* gc;  // grid coordinates: x [nx], then y [ny], then z [nz]
    // Vertices whose edge parameter t is within tau of 0 or 1 are the only ones
    // that can share a position with a vertex of another edge (mc_snap_tau).
    float tau;
    bool fma;  // arithmetic reading (iso::arith_fma at the call)
    int lgseg; // log2 of the point words per segment (the count kernel's CTA size times WPT)
};

// Workspace carved from one buffer (offsets 256-aligned).
struct McWs {
    uint32_t* S;                // sign bitmap [PW]
    uint32_t* info;             // per word: segment-local vertex offset | popc(ex) << 20 | popc(ey) << 26
    unsigned long long* blk;    // per segment of words: (V, F) sums, then exclusive offsets
    unsigned long long* vlist;  // vertex entries [capV]: pw | axis << 32 | bit << 34 | slot << 39
    unsigned long long* clist;  // cell entries [capF]: pw | bit << 32 | case << 37 | face offset << 45
    uint32_t* foff;             // per word with faces: segment-local face offset
    unsigned long long* ctr;    // [0] list size [1] snaps [2] barrier count [3] barrier gen [4] V' [5] F'
                                // [6] unused [7] scan ticket [8] merges [9] small hash full
                                // [10] cell entries [11] emit CTAs done
    unsigned long long* state;  // look-back state per segment (follows ctr; zeroed with it)
    uint32_t* small;            // SMALL_HC entries after the states (zeroed with them)
    float* gc;                  // grid coordinates [nx + ny + nz] (x, then y, then z)
    uint32_t* snaps;            // snapped vertex slots [capV]
    uint32_t* table;            // position hash of snapped vertices [HC]
    uint32_t* used;             // vertex used bits [capV / 32 + 1]
    uint32_t* newidx;           // compacted vertex index [capV]
    int32_t* ftmp;              // compacted faces [capF, 3]
    float* vtmp;                // compacted vertices [capV, 3]
    long long nBlk;             // segments at most (SEG_MIN point words each)
    uint32_t HC;
    size_t total;
};

constexpr uint32_t SMALL_HC = 1u << 15;  // merge-detection hash of emit (entries: vertex + 1, 0 = empty)
constexpr int NCTR = 16;
constexpr int WPT = 4;                       // point words per count thread
constexpr uint32_t SEG_MIN = 128 * WPT;      // words per segment (one scan entry) with 128-thread count CTAs

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

uint32_t hash_cap(long long capV) {
    uint32_t c = 1024;
    while ((long long)c < 2 * capV + 1024) c <<= 1;
    return c;
}

// Bytes cleared at the start of each call: counters, look-back states, small hash.
inline size_t zeroed_bytes(long long nBlk) { return size_t(NCTR) * 8 + size_t(nBlk) * 8 + size_t(SMALL_HC) * 4; }

McWs carve(int nx, int ny, int nz, long long capV, long long capF, uint8_t* base) {
    McWs w{};
    const long long NW = (nz + 31) / 32;
    const long long PW = (long long)nx * ny * NW;
    w.nBlk = (PW + SEG_MIN - 1) / SEG_MIN;  // segments at most (the smallest count CTA)
    w.HC = hash_cap(capV);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = base ? base + o : nullptr;
        o = al256(o + std::max<size_t>(bytes, 1));
        return p;
    };
    w.S = reinterpret_cast<uint32_t*>(take(size_t(PW) * 4));
    w.info = reinterpret_cast<uint32_t*>(take(size_t(PW) * 4));
    w.blk = reinterpret_cast<unsigned long long*>(take(size_t(w.nBlk + 1) * 16));
    w.vlist = reinterpret_cast<unsigned long long*>(take(size_t(capV) * 8));
    w.clist = reinterpret_cast<unsigned long long*>(take(size_t(capF) * 8));
    w.foff = reinterpret_cast<uint32_t*>(take(size_t(PW) * 4));
    w.ctr = reinterpret_cast<unsigned long long*>(take(zeroed_bytes(w.nBlk)));  // + states + small hash
    w.state = w.ctr ? w.ctr + NCTR : nullptr;
    w.small = w.ctr ? reinterpret_cast<uint32_t*>(w.state + w.nBlk) : nullptr;
    w.gc = reinterpret_cast<float*>(take(size_t(nx + ny + nz) * 4));
    w.snaps = reinterpret_cast<uint32_t*>(take(size_t(capV) * 4));
    w.table = reinterpret_cast<uint32_t*>(take(size_t(w.HC) * 4));
    w.used = reinterpret_cast<uint32_t*>(take(size_t(capV / 32 + 1) * 4));
    w.newidx = reinterpret_cast<uint32_t*>(take(size_t(capV) * 4));
    w.ftmp = reinterpret_cast<int32_t*>(take(size_t(capF) * 12));
    w.vtmp = reinterpret_cast<float*>(take(size_t(capV) * 12));
    w.total = o + 256;  // room to align the base
    return w;
}

// ---------------------------------------------------------------------------
// Per-word bit state.

// The 8 bitmap words around point word (x, y, w): s[dx][dy][0] = word w of row
// (x + dx, y + dy), s[..][1] = word w + 1 (0 past the row or grid).
struct Words {
    uint32_t s[2][2][2];
    int x, y, w;
    bool hasx, hasy;
};

__device__ __forceinline__ void load_words(const McGrid& g, const uint32_t* __restrict__ S, uint32_t pw, int x,
                                           int y, int w, Words& d) {
    d.x = x;
    d.y = y;
    d.w = w;
    d.hasx = x < g.nx - 1;
    d.hasy = y < g.ny - 1;
    const bool nxt = w + 1 < g.NW;
    const uint32_t sx = uint32_t(g.ny) * uint32_t(g.NW), sy = uint32_t(g.NW);
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const bool ok = (dx == 0 || d.hasx) && (dy == 0 || d.hasy);
            const uint32_t q = pw + dx * sx + dy * sy;
            d.s[dx][dy][0] = ok ? __ldg(S + q) : 0u;
            d.s[dx][dy][1] = (ok && nxt) ? __ldg(S + q + 1) : 0u;
        }
}

// Bits of word w whose z is below nz - 1 (z edges and cells need z + 1).
__device__ __forceinline__ uint32_t zmask(const McGrid& g, int w) {
    const int n = g.nz - 1 - 32 * w;
    return n >= 32 ? ~0u : (n <= 0 ? 0u : ((1u << n) - 1u));
}

// Word shifted so that bit b holds bit b + 1 (z + 1).
__device__ __forceinline__ uint32_t up1(uint32_t lo, uint32_t hi) { return __funnelshift_r(lo, hi, 1); }

__device__ __forceinline__ uint32_t ez_of(uint32_t lo, uint32_t hi, uint32_t zm) {
    return (lo ^ up1(lo, hi)) & zm;
}

// Active cells of the word: corners straddle the level.
__device__ __forceinline__ uint32_t active_cells(const Words& d, uint32_t zm) {
    if (!d.hasx || !d.hasy) return 0u;
    uint32_t a = ~0u, o = 0u;
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const uint32_t lo = d.s[dx][dy][0], hi = up1(lo, d.s[dx][dy][1]);
            a &= lo & hi;
            o |= lo | hi;
        }
    return (o & ~a) & zm;
}

// Case number of the cell at bit b: corner k = 4dx + 2dy + dz.
__device__ __forceinline__ uint32_t cell_case(const Words& d, int b) {
    uint32_t cs = 0;
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const uint32_t lo = d.s[dx][dy][0];
            const uint32_t hi = up1(lo, d.s[dx][dy][1]);
            cs |= ((lo >> b) & 1u) << (4 * dx + 2 * dy);
            cs |= ((hi >> b) & 1u) << (4 * dx + 2 * dy + 1);
        }
    return cs;
}

// Block-wide exclusive scan of two counts; totals in ta, tb.
template <int BLOCK>
__device__ __forceinline__ void block_scan2(uint32_t a, uint32_t b, uint32_t& ea, uint32_t& eb, uint32_t& ta,
                                            uint32_t& tb, uint32_t* sm) {
    constexpr int NWARP = BLOCK / 32;
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
// 2. count: one CTA per segment of CNT_THREADS * WPT point words (the CTA size
// is a launch parameter, "mc.count_threads"): per-word vertex entries,
// per-cell entries, and the segment's (V, F) sums, which mc_scan turns into
// offsets.

// Segment holding point word pw.
__device__ __forceinline__ uint32_t seg_of(const McGrid& g, uint32_t pw) { return pw >> g.lgseg; }

// (x, y, w) of point word pw.
__device__ __forceinline__ void word_xyw(const McGrid& g, uint32_t pw, int& x, int& y, int& w) {
    const uint32_t row = fdiv(pw, g.dNW);
    w = int(pw - row * uint32_t(g.NW));
    x = int(fdiv(row, g.dNY));
    y = int(row - uint32_t(x) * uint32_t(g.ny));
}

__device__ __forceinline__ void advance(const McGrid& g, int& x, int& y, int& w) {
    if (++w == g.NW) {
        w = 0;
        if (++y == g.ny) { y = 0; ++x; }
    }
}

__device__ __forceinline__ uint32_t pbits(float f) { return __float_as_uint(f == 0.0f ? 0.0f : f); }
__device__ __forceinline__ uint32_t phash(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}
__device__ __forceinline__ bool same_pos(const float* p, const float* q) {
    return p[0] == q[0] && p[1] == q[1] && p[2] == q[2];
}

// Position of the k-th (from 0) set bit of m; m has more than k set bits.
__device__ __forceinline__ int nth_set(uint32_t m, int k) {
    int base = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const uint32_t low = m & ((1u << s) - 1u);
        const int c = __popc(low);
        if (k >= c) { k -= c; m >>= s; base += s; }
        else m = low;
    }
    return base;
}

// Lane whose inclusive prefix first exceeds j (prefixes nondecreasing, j < total).
__device__ __forceinline__ int owner_of(uint32_t incl, uint32_t j) {
    int lo = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const uint32_t pv = __shfl_sync(~0u, incl, lo + s - 1);
        if (pv <= j) lo += s;
    }
    return lo;
}

template <int CNT_THREADS>
__global__ void __launch_bounds__(CNT_THREADS) mc_count(const McGrid g, const float amin0, const float amin1,
                                                        const float amin2, const float size0, const float size1,
                                                        const float size2, const uint32_t* __restrict__ S,
                                                        uint32_t* __restrict__ info,
                                                        unsigned long long* __restrict__ blk,
                                                        unsigned long long* __restrict__ vlist,
                                                        unsigned long long* __restrict__ clist,
                                                        uint32_t* __restrict__ foff, unsigned long long* ctr,
                                                        float* __restrict__ gc, const uint32_t nseg,
                                                        const long long capV, const long long capF) {
    constexpr uint32_t SEG = CNT_THREADS * WPT;  // words of the segment
    __shared__ uint32_t sm[64];
    __shared__ uint32_t nfs[SEG];  // faces of each word of the segment
    __shared__ uint32_t wcell[CNT_THREADS / 32], wvert[CNT_THREADS / 32];
    __shared__ unsigned long long cbase_s, vbase_s;
    __shared__ uint32_t nt4[64];  // triangle counts of the 256 cases, 4 per word
    __shared__ uint32_t vmask[3 * WPT][CNT_THREADS];  // x, y, z edge masks of each thread's words
    __shared__ uint32_t rows[4][WPT + 1][CNT_THREADS];  // sign words of rows (dx, dy), words k = 0..4
    iso::grid_wait();
    // grid coordinates (include/utils.cuh:62-80), read by the emit kernel
    const uint32_t gid = blockIdx.x * CNT_THREADS + threadIdx.x;
    const uint32_t ncoord = uint32_t(g.nx + g.ny + g.nz);
    if (gid < ncoord) {
        if (gid < uint32_t(g.nx)) gc[gid] = iso::grid_coord(gid, g.nx, amin0, size0, g.fma);
        else if (gid < uint32_t(g.nx + g.ny)) gc[gid] = iso::grid_coord(gid - g.nx, g.ny, amin1, size1, g.fma);
        else gc[gid] = iso::grid_coord(gid - g.nx - g.ny, g.nz, amin2, size2, g.fma);
    }
    const uint32_t seg = blockIdx.x;
    if (seg >= nseg) return;  // CTAs past the segments only write coordinates
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t sxw = uint32_t(g.ny) * uint32_t(g.NW), syw = uint32_t(g.NW);
    const bool vec = (g.NW & 3) == 0;  // rows start on 16-byte boundaries
    const uint32_t pw0 = seg * SEG + threadIdx.x * WPT;
#pragma unroll
    for (int k = 0; k < WPT; ++k) nfs[threadIdx.x * WPT + k] = 0u;
    if (threadIdx.x < 64) {
        const uint8_t* t = ISO_NTRI + g.method * 256 + 4 * threadIdx.x;
        nt4[threadIdx.x] = uint32_t(t[0]) | (uint32_t(t[1]) << 8) | (uint32_t(t[2]) << 16) | (uint32_t(t[3]) << 24);
    }
    // bitmap words pw0 .. pw0 + 3 of the rows (x, y), (x, y+1), (x+1, y), (x+1, y+1)
    uint32_t r[2][2][WPT];
    int x = 0, y = 0, w = 0;
    if (pw0 < g.PW) word_xyw(g, pw0, x, y, w);
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            const uint32_t q = pw0 + dx * sxw + dy * syw;
            if (vec && pw0 + WPT <= g.PW && q + WPT <= g.PW) {
                const uint4 v4 = __ldg(reinterpret_cast<const uint4*>(S + q));
                r[dx][dy][0] = v4.x; r[dx][dy][1] = v4.y; r[dx][dy][2] = v4.z; r[dx][dy][3] = v4.w;
            } else {
#pragma unroll
                for (int k = 0; k < WPT; ++k) r[dx][dy][k] = (q + k < g.PW) ? __ldg(S + q + k) : 0u;
            }
        }
    // word pw0 + 4 of each row: the next lane's first word, or a load
    uint32_t nx4[2][2];
#pragma unroll
    for (int dx = 0; dx < 2; ++dx)
#pragma unroll
        for (int dy = 0; dy < 2; ++dy) {
            nx4[dx][dy] = __shfl_down_sync(~0u, r[dx][dy][0], 1);
            if (lane == 31) {
                const uint32_t q = pw0 + WPT + dx * sxw + dy * syw;
                nx4[dx][dy] = q < g.PW ? __ldg(S + q) : 0u;
            }
        }
    uint32_t nv[WPT], cxy[WPT], act[WPT];
#pragma unroll
    for (int k = 0; k < WPT; ++k) { nv[k] = 0; cxy[k] = 0; act[k] = 0; }
    // Most words lie wholly inside or outside the surface: the word and its
    // grid neighbours' words are all 0 or all ~0, and nothing crosses.  A warp
    // whose 128 words are all like that skips the rest.
    bool quiet_all;
    {
        // conservative: all 20 loaded words equal, and all 0 or all ~0 (words at
        // the grid's edges may fail it and take the exact path)
        const uint32_t u = r[0][0][0];
        uint32_t diff = 0;
#pragma unroll
        for (int dx = 0; dx < 2; ++dx)
#pragma unroll
            for (int dy = 0; dy < 2; ++dy) {
                diff |= nx4[dx][dy] ^ u;
#pragma unroll
                for (int k = 0; k < WPT; ++k) diff |= r[dx][dy][k] ^ u;
            }
        quiet_all = (u == 0u || u == ~0u) && diff == 0u;
    }
    const bool warp_quiet = __all_sync(~0u, quiet_all);
    if (!warp_quiet) {
        // the cells of these words read their corners from here
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int k = 0; k < WPT; ++k) rows[q][k][threadIdx.x] = r[q >> 1][q & 1][k];
            rows[q][WPT][threadIdx.x] = nx4[q >> 1][q & 1];
        }
#pragma unroll
        for (int k = 0; k < WPT; ++k) {
            if (pw0 + k < g.PW) {
                Words d;
                d.x = x; d.y = y; d.w = w;
                d.hasx = x < g.nx - 1;
                d.hasy = y < g.ny - 1;
                const bool nxt = w + 1 < g.NW;
#pragma unroll
                for (int dx = 0; dx < 2; ++dx)
#pragma unroll
                    for (int dy = 0; dy < 2; ++dy) {
                        const bool ok = (dx == 0 || d.hasx) && (dy == 0 || d.hasy);
                        d.s[dx][dy][0] = ok ? r[dx][dy][k] : 0u;
                        d.s[dx][dy][1] = (ok && nxt) ? (k + 1 < WPT ? r[dx][dy][(k + 1) % WPT] : nx4[dx][dy]) : 0u;
                    }
                const uint32_t zm = zmask(g, w);
                const uint32_t ex = d.hasx ? (d.s[0][0][0] ^ d.s[1][0][0]) : 0u;
                const uint32_t ey = d.hasy ? (d.s[0][0][0] ^ d.s[0][1][0]) : 0u;
                const uint32_t ez = ez_of(d.s[0][0][0], d.s[0][0][1], zm);
                nv[k] = __popc(ex) + __popc(ey) + __popc(ez);
                cxy[k] = (uint32_t(__popc(ex)) << 20) | (uint32_t(__popc(ey)) << 26);
                act[k] = active_cells(d, zm);
                vmask[3 * k][threadIdx.x] = ex;
                vmask[3 * k + 1][threadIdx.x] = ey;
                vmask[3 * k + 2][threadIdx.x] = ez;
                advance(g, x, y, w);
            }
        }
    }
    // nfs cleared.  A segment whose warps are all quiet has no crossed edge and
    // no active cell: its sums are 0, and no cell reads its words' vertex
    // offsets (a cell's edges lie in words with crossings), so it stops here.
    if (!__syncthreads_or(!warp_quiet)) {
        if (threadIdx.x == 0) {
            blk[2 * seg] = 0ull;
            blk[2 * seg + 1] = 0ull;
        }
        return;
    }
    uint32_t sv = 0;
#pragma unroll
    for (int k = 0; k < WPT; ++k) sv += nv[k];
    // active cells, one per lane of the warp: triangle counts, and a cell entry
    // with the cell's face offset within its word (cells of a word come in bit
    // order: a segmented scan over the lanes plus the word's faces of earlier rounds)
    {
        const uint32_t na = __popc(act[0]) + __popc(act[1]) + __popc(act[2]) + __popc(act[3]);
        uint32_t incl = na, vsum = sv;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            const uint32_t t = __shfl_up_sync(~0u, incl, dd);
            if (lane >= dd) incl += t;
            vsum += __shfl_xor_sync(~0u, vsum, dd);
        }
        const uint32_t total = __shfl_sync(~0u, incl, 31);
        // the CTA's cell entries and vertex entries are allocated at once: warp
        // offsets, one atomic each, both in flight together
        if (lane == 0) {
            wcell[warp] = total;
            wvert[warp] = vsum;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int q = 0; q < CNT_THREADS / 32; ++q) {
                const uint32_t c = wcell[q];
                wcell[q] = run;
                run += c;
            }
            cbase_s = run ? atomicAdd(ctr + 10, (unsigned long long)run) : 0ull;
        } else if (threadIdx.x == 32) {
            uint32_t run = 0;
            for (int q = 0; q < CNT_THREADS / 32; ++q) run += wvert[q];
            vbase_s = run ? atomicAdd(ctr, (unsigned long long)run) : 0ull;
        }
        __syncthreads();
        const unsigned long long wbase = cbase_s + wcell[warp];
        for (uint32_t rr = 0; rr < total; rr += 32) {
            const uint32_t j = rr + lane;
            const int o = owner_of(incl, j);
            const uint32_t oexcl = __shfl_sync(~0u, incl - na, o);
            uint32_t oa[WPT];
#pragma unroll
            for (int k = 0; k < WPT; ++k) oa[k] = __shfl_sync(~0u, act[k], o);
            const bool valid = j < total;
            uint32_t wid = 0xffffffffu, ntc = 0, cs = 0, pw = 0;
            int b = 0;
            if (valid) {
                int kk = int(j - oexcl), k = 0;
                uint32_t m = oa[0];
#pragma unroll
                for (int q = 0; q < WPT - 1; ++q) {
                    const int c = __popc(m);
                    if (kk >= c) { kk -= c; m = oa[q + 1]; k = q + 1; }
                    else break;
                }
                b = nth_set(m, kk);
                const uint32_t ot = uint32_t(warp * 32 + o);
                wid = ot * WPT + uint32_t(k);
                pw = seg * SEG + wid;
                // corners from the owner's row words (an active cell has rows
                // x + 1 and y + 1, and z + 1 in word w + 1 only at bit 31)
                Words d;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    d.s[q >> 1][q & 1][0] = rows[q][k][ot];
                    d.s[q >> 1][q & 1][1] = rows[q][k + 1][ot];
                }
                cs = cell_case(d, b);
                ntc = (nt4[cs >> 2] >> (8 * (cs & 3))) & 0xffu;
            }
            uint32_t sc = ntc;
#pragma unroll
            for (int dd = 1; dd < 32; dd <<= 1) {
                const uint32_t t = __shfl_up_sync(~0u, sc, dd);
                if (lane >= dd) sc += t;
            }
            const uint32_t prev_wid = __shfl_up_sync(~0u, wid, 1);
            const uint32_t next_wid = __shfl_down_sync(~0u, wid, 1);
            const uint32_t heads = __ballot_sync(~0u, valid && (lane == 0 || prev_wid != wid));
            const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
            const uint32_t base = __shfl_sync(~0u, sc, start > 0 ? start - 1 : 0);
            const uint32_t within_round = sc - ntc - (start > 0 ? base : 0u);
            const uint32_t carry = valid ? nfs[wid] : 0u;
            __syncwarp();
            if (valid) {
                const unsigned long long ci = wbase + j;
                if ((long long)ci < capF)
                    clist[ci] = (unsigned long long)pw | ((unsigned long long)b << 32) |
                                ((unsigned long long)cs << 37) |
                                ((unsigned long long)(carry + within_round) << 45);
                const bool tail = lane == 31 || next_wid != wid;
                if (tail) nfs[wid] = carry + within_round + ntc;
            }
            __syncwarp();
        }
    }
    __syncthreads();
    uint32_t nf[WPT], sf = 0;
#pragma unroll
    for (int k = 0; k < WPT; ++k) {
        nf[k] = nfs[threadIdx.x * WPT + k];
        sf += nf[k];
    }
    uint32_t ev, ef, tv, tf;
    block_scan2<CNT_THREADS>(sv, sf, ev, ef, tv, tf, sm);
    // vertex entries: the CTA's block of entries (allocated above), each entry
    // at the block base plus its segment-local slot (x edges, then y, then z of
    // each word); one vertex per lane of the warp, so consecutive lanes store
    // consecutive entries
    const unsigned long long vb0 = vbase_s;
    {
        uint32_t incl = sv;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            const uint32_t t = __shfl_up_sync(~0u, incl, dd);
            if (lane >= dd) incl += t;
        }
        const uint32_t total = __shfl_sync(~0u, incl, 31);
        for (uint32_t rr = 0; rr < total; rr += 32) {
            const uint32_t j = rr + lane;
            const int o = owner_of(incl, j);
            const uint32_t oexcl = __shfl_sync(~0u, incl - sv, o);
            const uint32_t oev = __shfl_sync(~0u, ev, o);
            uint32_t onv[WPT];
#pragma unroll
            for (int k = 0; k < WPT; ++k) onv[k] = __shfl_sync(~0u, nv[k], o);
            if (j < total) {
                uint32_t kk = j - oexcl, slot = oev + kk;
                int k = 0;
#pragma unroll
                for (int q = 0; q < WPT - 1; ++q) {
                    if (k == q && kk >= onv[q]) { kk -= onv[q]; k = q + 1; }
                }
                const uint32_t ot = uint32_t(warp * 32 + o);
                const uint32_t m0 = vmask[3 * k][ot], m1 = vmask[3 * k + 1][ot], m2 = vmask[3 * k + 2][ot];
                const uint32_t c0 = __popc(m0), c1 = __popc(m1);
                int ax, bb;
                if (kk < c0) { ax = 0; bb = nth_set(m0, int(kk)); }
                else if (kk < c0 + c1) { ax = 1; bb = nth_set(m1, int(kk - c0)); }
                else { ax = 2; bb = nth_set(m2, int(kk - c0 - c1)); }
                const uint32_t pw = seg * SEG + ot * WPT + uint32_t(k);
                const unsigned long long vb = vb0 + slot;
                if ((long long)vb < capV)
                    vlist[vb] = (unsigned long long)pw | ((unsigned long long)ax << 32) |
                                ((unsigned long long)bb << 34) | ((unsigned long long)slot << 39);
            }
        }
    }
    if (vec && pw0 + WPT <= g.PW) {
        *reinterpret_cast<uint4*>(info + pw0) =
            make_uint4(ev | cxy[0], (ev + nv[0]) | cxy[1], (ev + nv[0] + nv[1]) | cxy[2],
                       (ev + nv[0] + nv[1] + nv[2]) | cxy[3]);
    }
#pragma unroll
    for (int k = 0; k < WPT; ++k) {
        const uint32_t pw = pw0 + k;
        if (pw < g.PW) {
            if (!(vec && pw0 + WPT <= g.PW)) info[pw] = ev | cxy[k];
            if (nf[k]) foff[pw] = ef;
        }
        ev += nv[k];
        ef += nf[k];
    }
    if (threadIdx.x == 0) {
        blk[2 * seg] = tv;
        blk[2 * seg + 1] = tf;
    }
}

// ---------------------------------------------------------------------------
// 3. scan of the per-segment (V, F) sums of mc_count into exclusive offsets:
// CTAs take chunks of SCAN_PER * SCAN_THREADS segments in ticket order and chain
// their totals by decoupled look-back.  The last chunk writes the totals and
// checks the capacities.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER = 1;

__global__ void __launch_bounds__(SCAN_THREADS) mc_scan(unsigned long long* blk, uint32_t nseg,
                                                        unsigned long long* ctr, unsigned long long* state,
                                                        long long* counts, int* status, long long capV,
                                                        long long capF) {
    __shared__ uint32_t sm[64];
    __shared__ uint32_t chunk_s;
    __shared__ unsigned long long pre_s[2];
    iso::grid_wait();
    if (threadIdx.x == 0) chunk_s = uint32_t(atomicAdd(ctr + 7, 1ull));
    __syncthreads();
    const uint32_t chunk = chunk_s;
    const uint32_t nchunk = (nseg + SCAN_PER * SCAN_THREADS - 1) / (SCAN_PER * SCAN_THREADS);
    const uint32_t s0 = chunk * SCAN_PER * SCAN_THREADS + threadIdx.x * SCAN_PER;
    uint32_t a[SCAN_PER], b[SCAN_PER], sa = 0, sb = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        a[k] = s0 + k < nseg ? uint32_t(blk[2 * (s0 + k)]) : 0u;
        b[k] = s0 + k < nseg ? uint32_t(blk[2 * (s0 + k) + 1]) : 0u;
        sa += a[k];
        sb += b[k];
    }
    uint32_t ea, eb, ta, tb;
    block_scan2<SCAN_THREADS>(sa, sb, ea, eb, ta, tb, sm);
    if (threadIdx.x < 32) {
        unsigned long long pv = 0, pf = 0;
        if (chunk == 0) {
            if (threadIdx.x == 0) atomicExch(state, lb_pack(LB_INC, ta, tb));
        } else {
            if (threadIdx.x == 0) atomicExch(state + chunk, lb_pack(LB_AGG, ta, tb));
            look_back(state, chunk, pv, pf, status);
            if (threadIdx.x == 0) atomicExch(state + chunk, lb_pack(LB_INC, pv + ta, pf + tb));
        }
        if (threadIdx.x == 0) {
            pre_s[0] = pv;
            pre_s[1] = pf;
            if (chunk == nchunk - 1) {
                const unsigned long long V = pv + ta, F = pf + tb;
                counts[0] = (long long)V;
                counts[1] = (long long)F;
                if ((long long)V > capV || (long long)F > capF || V >= LB_MASK31 || F >= LB_MASK31)
                    atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
            }
        }
    }
    __syncthreads();
    unsigned long long ov = pre_s[0] + ea, of = pre_s[1] + eb;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        if (s0 + k < nseg) {
            blk[2 * (s0 + k)] = ov;
            blk[2 * (s0 + k) + 1] = of;
        }
        ov += a[k];
        of += b[k];
    }
}

// The scan's look-back for chunk `seg` over states nobody publishes: it must
// give up after `limit` polls and set the status (a test of the bounded wait).
__global__ void lookback_probe(unsigned long long* state, uint32_t seg, uint32_t limit, int* status,
                               unsigned long long* out) {
    unsigned long long ev = 0, ef = 0;
    look_back(state, seg, ev, ef, status, limit);
    if (threadIdx.x == 0) {
        out[0] = ev;
        out[1] = ef;
    }
}

// ---------------------------------------------------------------------------
// 4. emit: one thread per vertex entry, then one thread per cell entry.

__device__ __forceinline__ float gx(const McGrid& g, int x) { return g.gc[x]; }
__device__ __forceinline__ float gy(const McGrid& g, int y) { return g.gc[g.nx + y]; }
__device__ __forceinline__ float gz(const McGrid& g, int z) { return g.gc[g.nx + g.ny + z]; }

struct EmitArgs {
    const float* vals;
    const uint32_t* S;
    const uint32_t* info;
    const unsigned long long* blk;
    const uint32_t* foff;
    const unsigned long long* vlist;
    const unsigned long long* clist;
    unsigned long long* ctr;
    uint32_t* snaps;
    uint32_t* small;
    float* vout;
    int32_t* fout;
    long long* counts;
    int* status;
    long long capV, capF;
    unsigned nbv;  // CTAs with the vertex role; the rest emit faces
    McWs w;        // for the fix-up
    long long* vedge;  // optional: each vertex's grid edge
};

// Vertex role: one thread per vertex entry; CTA `bi` of `nb`.
template <int EMIT_THREADS>
__device__ void emit_vertices(const McGrid& g, const EmitArgs& a, unsigned bi, unsigned nb) {
    const float* __restrict__ vals = a.vals;
    const unsigned long long* __restrict__ blk = a.blk;
    const unsigned long long* __restrict__ vlist = a.vlist;
    unsigned long long* ctr = a.ctr;
    uint32_t* __restrict__ snaps = a.snaps;
    uint32_t* small = a.small;
    float* vout = a.vout;
    const long long capV = a.capV;
    const unsigned long long n = min(ctr[0], (unsigned long long)capV);
    const long long sxv = (long long)g.ny * g.nz;
    for (unsigned long long i = (unsigned long long)bi * EMIT_THREADS + threadIdx.x; i < n;
         i += (unsigned long long)nb * EMIT_THREADS) {
        const unsigned long long e = vlist[i];
        const uint32_t pw = uint32_t(e);
        const int ax = int((e >> 32) & 3u), b = int((e >> 34) & 31u);
        const uint32_t vi = uint32_t(blk[2 * seg_of(g, pw)]) + uint32_t((e >> 39) & 0xfffffu);
        int x, y, w;
        word_xyw(g, pw, x, y, w);
        const int z = 32 * w + b;
        const long long ia = ((long long)x * g.ny + y) * g.nz + z;
        const long long step = ax == 0 ? sxv : (ax == 1 ? (long long)g.nz : 1ll);
        const float va = __ldg(vals + ia), vb = __ldg(vals + ia + step);
        const float t = iso::cross_t(g.level, va, vb);
        const float xa = gx(g, x), ya = gy(g, y), za = gz(g, z);
        const float xb = ax == 0 ? gx(g, x + 1) : xa;
        const float yb = ax == 1 ? gy(g, y + 1) : ya;
        const float zb = ax == 2 ? gz(g, z + 1) : za;
        const float px = iso::lerp1(t, xa, xb, g.fma), py = iso::lerp1(t, ya, yb, g.fma),
                    pz = iso::lerp1(t, za, zb, g.fma);
        float* vo = vout + 3ll * vi;
        vo[0] = px;
        vo[1] = py;
        vo[2] = pz;
        if (a.vedge) a.vedge[vi] = 3 * ia + ax;
        if (!(t >= g.tau && t <= 1.0f - g.tau) || (px == xa && py == ya && pz == za) ||
            (px == xb && py == yb && pz == zb)) {
            // a candidate for sharing its position: list it, and look for an
            // equal position among the candidates so far
            const unsigned long long sidx = atomicAdd(ctr + 1, 1ull);
            if ((long long)sidx < capV) snaps[sidx] = vi;
            __threadfence();  // the position is visible before the hash entry
            uint32_t h = phash(pbits(px), pbits(py), pbits(pz)) & (SMALL_HC - 1u);
            bool placed = false;
            for (uint32_t probe = 0; probe < SMALL_HC; ++probe, h = (h + 1) & (SMALL_HC - 1u)) {
                const uint32_t cur = atomicCAS(&small[h], 0u, vi + 1u);
                if (cur == 0u) { placed = true; break; }
                if (same_pos(vo, vout + 3ll * (cur - 1u))) {
                    atomicAdd(ctr + 8, 1ull);
                    placed = true;
                    break;
                }
            }
            if (!placed) atomicOr(reinterpret_cast<unsigned int*>(ctr + 9), 1u);
        }
    }
}

// Face role: one thread per cell entry; CTA `bi` of `nb`.
template <int EMIT_THREADS>
__device__ void emit_faces(const McGrid& g, const EmitArgs& a, unsigned bi, unsigned nb) {
    __shared__ unsigned long long tpk[256];  // packed triangle lists of the table
    __shared__ uint16_t est[256];
    __shared__ uint32_t vid[12][EMIT_THREADS];
    const uint32_t* __restrict__ S = a.S;
    const uint32_t* __restrict__ info = a.info;
    const unsigned long long* __restrict__ blk = a.blk;
    const uint32_t* __restrict__ foff = a.foff;
    const unsigned long long* __restrict__ clist = a.clist;
    int32_t* __restrict__ fout = a.fout;
    for (int i = threadIdx.x; i < 256; i += EMIT_THREADS) {
        tpk[i] = ISO_TRI_PACKED[g.method * 256 + i];
        est[i] = ISO_EDGE_STATUS[i];
    }
    __syncthreads();
    const unsigned long long n = min(a.ctr[10], (unsigned long long)a.capF);
    const uint32_t sxw = uint32_t(g.ny) * uint32_t(g.NW);
    const int tid = threadIdx.x;
    for (unsigned long long i = (unsigned long long)bi * EMIT_THREADS + tid; i < n;
         i += (unsigned long long)nb * EMIT_THREADS) {
        const unsigned long long e = clist[i];
        const uint32_t pw = uint32_t(e);
        const int b = int((e >> 32) & 31u);
        const uint32_t cs = uint32_t((e >> 37) & 255u);
        int x, y, w;
        word_xyw(g, pw, x, y, w);
        const unsigned long long fo = blk[2 * seg_of(g, pw) + 1] + foff[pw] + ((e >> 45) & 255u);
        Words d;
        load_words(g, S, pw, x, y, w, d);
        const uint32_t zm = zmask(g, w);
        const uint32_t es = est[cs];
        const int hi = (b + 1) >> 5;  // the cell's z + 1 lies in word w + 1
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            if (!((es >> k) & 1u)) continue;
            const int a = iso_edge_corner(2 * k), c = iso_edge_corner(2 * k + 1);
            const int ax = (c - a) == 4 ? 0 : ((c - a) == 2 ? 1 : 2);
            const int adx = a >> 2, ady = (a >> 1) & 1, adz = a & 1;
            const int ww = adz ? hi : 0;
            const int bit = (b + adz) & 31;
            uint32_t m;
            if (ax == 0) m = ww ? (d.s[0][ady][1] ^ d.s[1][ady][1]) : (d.s[0][ady][0] ^ d.s[1][ady][0]);
            else if (ax == 1) m = ww ? (d.s[adx][0][1] ^ d.s[adx][1][1]) : (d.s[adx][0][0] ^ d.s[adx][1][0]);
            else m = ez_of(d.s[adx][ady][0], d.s[adx][ady][1], zm);
            const uint32_t q = pw + uint32_t(adx) * sxw + uint32_t(ady) * uint32_t(g.NW) + uint32_t(ww);
            const uint32_t inf = info[q];
            uint32_t off = uint32_t(blk[2 * seg_of(g, q)]) + (inf & 0xfffffu);
            if (ax >= 1) off += (inf >> 20) & 63u;
            if (ax == 2) off += (inf >> 26) & 63u;
            vid[k][tid] = off + __popc(m & ((1u << bit) - 1u));
        }
        unsigned long long pk = tpk[cs];
        const int ntc = int(pk >> 60);
        int32_t* f3 = fout + 3 * fo;
        for (int k = 0; k < ntc; ++k, pk >>= 12, f3 += 3) {
            f3[0] = int32_t(vid[pk & 15u][tid]);
            f3[1] = int32_t(vid[(pk >> 4) & 15u][tid]);
            f3[2] = int32_t(vid[(pk >> 8) & 15u][tid]);
        }
    }
}

__device__ void fixup_block(const McWs& w, float* vout, int32_t* fout, long long* counts, int* status,
                            long long capV, long long* vedge);

template <int EMIT_THREADS>
__global__ void __launch_bounds__(EMIT_THREADS) mc_emit(const McGrid g, const EmitArgs a) {
    __shared__ int last;
    iso::grid_wait();
    if (a.counts[0] > a.capV || a.counts[1] > a.capF || a.counts[0] > 0x7fffffffll) return;
    if (blockIdx.x < a.nbv) emit_vertices<EMIT_THREADS>(g, a, blockIdx.x, a.nbv);
    else emit_faces<EMIT_THREADS>(g, a, blockIdx.x - a.nbv, gridDim.x - a.nbv);
    // the last CTA to finish sees every vertex and face; it does the fix-up if
    // the emit found coinciding positions
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(a.ctr + 11, 1ull) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (a.ctr[1] == 0 || (a.ctr[8] == 0 && a.ctr[9] == 0)) return;
    fixup_block(a.w, a.vout, a.fout, a.counts, a.status, a.capV, a.vedge);
}

// ---------------------------------------------------------------------------
// 4. fix-up: run by the last CTA of mc_emit to finish, and only when some vertex
// positions coincide (found by the emit kernel's small hash).  It merges the
// candidates by exact position (smallest index wins, as a sorted weld keeps the
// first), drops faces that became degenerate and compacts vertices and faces,
// keeping their order.  One CTA: these inputs are rare (values exactly at the
// level on grid points, or grids near float resolution).

__device__ __forceinline__ bool face_keep(const int32_t* f) {
    return f[0] != f[1] && f[0] != f[2] && f[1] != f[2];
}

// Exclusive block scan of one count; total in `total`.
__device__ __forceinline__ uint32_t block_excl(uint32_t x, uint32_t& total, uint32_t* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t u = __shfl_up_sync(~0u, inc, d);
        if (lane >= d) inc += u;
    }
    if (lane == 31) sm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t y = lane < nwarps ? sm[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, y, d);
            if (lane >= d) y += u;
        }
        sm[lane] = y;
    }
    __syncthreads();
    const uint32_t ex = (warp ? sm[warp - 1] : 0u) + inc - x;
    total = sm[31];
    __syncthreads();
    return ex;
}

// Smallest index of a snapped vertex at vertex v's position, or v.
__device__ uint32_t rep_of(const McWs& w, const float* vout, uint32_t v) {
    const float* p = vout + 3ll * v;
    const uint32_t mask = w.HC - 1;
    uint32_t h = phash(pbits(p[0]), pbits(p[1]), pbits(p[2])) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const uint32_t j = w.table[h];
        if (j == 0xffffffffu) break;
        if (same_pos(p, vout + 3ll * j)) return j;
    }
    return v;
}

__device__ void fixup_block(const McWs& w, float* vout, int32_t* fout, long long* counts, int* status,
                            long long capV, long long* vedge) {
    __shared__ uint32_t sm[32];
    const long long V = counts[0], F = counts[1];
    const long long nsnap = min((long long)w.ctr[1], capV);
    const uint32_t mask = w.HC - 1;
    const int T = blockDim.x, tid = threadIdx.x;
    for (long long i = tid; i < w.HC; i += T) w.table[i] = 0xffffffffu;
    for (long long i = tid; i < V / 32 + 1; i += T) w.used[i] = 0u;
    __syncthreads();
    // candidates into the position hash; the smallest index wins
    for (long long s = tid; s < nsnap; s += T) {
        const uint32_t v = w.snaps[s];
        const float* p = vout + 3ll * v;
        uint32_t h = phash(pbits(p[0]), pbits(p[1]), pbits(p[2])) & mask;
        bool done = false;
        for (uint32_t probe = 0; probe <= mask && !done; ++probe, h = (h + 1) & mask) {
            const uint32_t cur = atomicCAS(&w.table[h], 0xffffffffu, v);
            if (cur == 0xffffffffu) { done = true; break; }
            if (same_pos(p, vout + 3ll * cur)) {
                atomicMin(&w.table[h], v);
                done = true;
            }
        }
        if (!done) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
    }
    __syncthreads();
    // faces: merge, keep the non-degenerate ones in order, mark their vertices
    uint32_t fn = 0;
    for (long long base = 0; base < F; base += T) {
        const long long f = base + tid;
        uint32_t keep = 0;
        int32_t v3[3] = {0, 0, 0};
        if (f < F) {
#pragma unroll
            for (int k = 0; k < 3; ++k) v3[k] = int32_t(rep_of(w, vout, uint32_t(fout[3 * f + k])));
            keep = face_keep(v3);
        }
        uint32_t tot;
        const uint32_t ex = block_excl(keep, tot, sm);
        if (keep) {
            int32_t* o = w.ftmp + 3ll * (fn + ex);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                o[k] = v3[k];
                atomicOr(&w.used[uint32_t(v3[k]) >> 5], 1u << (uint32_t(v3[k]) & 31u));
            }
        }
        fn += tot;
    }
    __syncthreads();
    // vertices still used, in order
    uint32_t vn = 0;
    for (long long base = 0; base < V; base += T) {
        const long long v = base + tid;
        const uint32_t u = v < V ? (w.used[v >> 5] >> (v & 31)) & 1u : 0u;
        // edges move in place: every read of this window precedes the scan's
        // barriers, and a vertex never moves to a higher index
        const long long ev = (u && vedge) ? vedge[v] : 0;
        uint32_t tot;
        const uint32_t ex = block_excl(u, tot, sm);
        if (u) {
            const uint32_t j = vn + ex;
            if (vedge) vedge[j] = ev;
            w.newidx[v] = j;
            w.vtmp[3ll * j] = vout[3 * v];
            w.vtmp[3ll * j + 1] = vout[3 * v + 1];
            w.vtmp[3ll * j + 2] = vout[3 * v + 2];
        }
        vn += tot;
    }
    __syncthreads();
    for (long long j = tid; j < 3ll * vn; j += T) vout[j] = w.vtmp[j];
    for (long long j = tid; j < 3ll * fn; j += T) fout[j] = int32_t(w.newidx[w.ftmp[j]]);
    if (tid == 0) {
        counts[0] = vn;
        counts[1] = fn;
    }
}

// ---------------------------------------------------------------------------
// 1. sign bitmap

constexpr int SIGN_BLOCK = 256;
constexpr int SIGN_UNROLL = 16;

// Bit z % 32 of word [(x * ny + y) * NWg + z / 32] is (v - level < 0).  One warp
// per grid row, all of the row's loads in flight before the ballots; lane w
// keeps word w so each 32 words leave in one store.
__global__ void __launch_bounds__(SIGN_BLOCK) mc_signs(const float* __restrict__ vals, long long rows,
                                                       int nz, float level, uint32_t* __restrict__ out,
                                                       unsigned long long* __restrict__ zero, long long nzero) {
    iso::grid_wait();
    // counters, look-back states and the small hash of the call start at zero
    for (long long i = (long long)blockIdx.x * SIGN_BLOCK + threadIdx.x; i < nzero;
         i += (long long)gridDim.x * SIGN_BLOCK)
        zero[i] = 0ull;
    const int lane = threadIdx.x & 31;
    const int NWg = (nz + 31) / 32;
    const long long warps = (long long)gridDim.x * (SIGN_BLOCK / 32);
    for (long long row = (long long)blockIdx.x * (SIGN_BLOCK / 32) + (threadIdx.x >> 5); row < rows;
         row += warps) {
        const float* rp = vals + row * nz;
        uint32_t* op = out + row * NWg;
        for (int wb = 0; wb < NWg; wb += 32) {
            uint32_t mine = 0;
            for (int w0 = wb; w0 < min(NWg, wb + 32); w0 += SIGN_UNROLL) {
                float v[SIGN_UNROLL];
#pragma unroll
                for (int u = 0; u < SIGN_UNROLL; ++u) {
                    const int z = 32 * (w0 + u) + lane;
                    v[u] = (w0 + u < NWg && z < nz) ? __ldcs(rp + z) : level;  // read once: evict first
                }
#pragma unroll
                for (int u = 0; u < SIGN_UNROLL; ++u) {
                    const uint32_t b = __ballot_sync(~0u, iso::below(v[u], level));
                    if (((w0 + u) & 31) == lane) mine = b;
                }
            }
            if (wb + lane < NWg) op[wb + lane] = mine;
        }
    }
}

std::mutex g_mu;
int g_block = 256;

int sm_count() {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

template <int EMIT_THREADS>
int launch_emit(const McParams& p, const McGrid& g, const McWs& w, cudaStream_t st, int sms) {
    static int per = -1;
    if (per < 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mc_emit<EMIT_THREADS>, EMIT_THREADS, 0);
    // entries are a fraction of the capacities; the loops are grid-stride.  The
    // resident CTAs are split between the roles in proportion to the work
    // (a vertex costs about half a cell).
    const long long resident = (long long)sms * std::max(per, 1);
    const auto want = [&](long long cap) { return std::max<long long>(1, (cap + EMIT_THREADS - 1) / EMIT_THREADS); };
    const long long nbv = std::max<long long>(1, std::min(want(p.capV), resident / 3));
    const long long nbf = std::max<long long>(1, std::min(want(p.capF), resident - nbv));
    EmitArgs a{p.vals, w.S, w.info, w.blk, w.foff, w.vlist, w.clist, w.ctr, w.snaps, w.small,
               p.vout, p.fout, p.counts, p.status, p.capV, p.capF, unsigned(nbv), w, p.vedge};
    {
        iso::ProfScope ps("mc_emit", st);
        iso::launch_pdl(mc_emit<EMIT_THREADS>, unsigned(nbv + nbf), EMIT_THREADS, st, g, a);
        if (cudaGetLastError() != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    }
    return 0;
}

int launch_count_emit(const McParams& p, const McGrid& g, const McWs& w, cudaStream_t st) {
    const int sms = sm_count();
    {
        iso::ProfScope ps("mc_count", st);
        const long long ncoord = (long long)p.nx + p.ny + p.nz;
        const int ct = 1 << (g.lgseg - 2);  // the count CTA's threads (WPT = 4 words each)
        const long long nseg = (g.PW + (1ll << g.lgseg) - 1) >> g.lgseg;
        const long long grid = std::max<long long>(nseg, (ncoord + ct - 1) / ct);
        iso::launch_pdl(ct == 128 ? mc_count<128> : mc_count<256>, unsigned(grid), unsigned(ct), st, g, p.amin[0],
                        p.amin[1], p.amin[2], p.asize[0], p.asize[1], p.asize[2], w.S, w.info, w.blk, w.vlist, w.clist,
                        w.foff, w.ctr, w.gc, uint32_t(nseg), p.capV, p.capF);
        if (cudaGetLastError() != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    }
    {
        iso::ProfScope ps("mc_scan", st);
        const uint32_t nseg = uint32_t((g.PW + (1ll << g.lgseg) - 1) >> g.lgseg);
        const uint32_t nchunk = (nseg + SCAN_PER * SCAN_THREADS - 1) / (SCAN_PER * SCAN_THREADS);
        iso::launch_pdl(mc_scan, nchunk, SCAN_THREADS, st, w.blk, nseg, w.ctr, w.state, p.counts, p.status, p.capV,
                   p.capF);
        if (cudaGetLastError() != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    }
    const int block = mc_get_block();
    return block == 128 ? launch_emit<128>(p, g, w, st, sms) : launch_emit<256>(p, g, w, st, sms);
}

}  // namespace

int mc_set_block(int threads) {
    if (threads != 128 && threads != 256) return iso::fail_code(ISO_ERR_ARG);
    std::lock_guard<std::mutex> lk(g_mu);
    g_block = threads;
    return 0;
}

int mc_get_block() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_block;
}

void mc_signs_launch(const float* vals, int nx, int ny, int nz, float level, uint32_t* out,
                     cudaStream_t st, unsigned long long* zero, long long nzero) {
    const long long rows = (long long)nx * ny;
    const long long want = (rows + (SIGN_BLOCK / 32) - 1) / (SIGN_BLOCK / 32);
    const long long per = iso::tune_get(iso::TUNE_MC_SIGN_CTAS);
    const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sm_count() * per));
    iso::launch_pdl(mc_signs, unsigned(grid), SIGN_BLOCK, st, vals, rows, nz, level, out, zero, nzero);
}

// Bound on t for an edge vertex to land within a few ulps of an endpoint (the
// only place two edges' vertices can meet).  The lerp (1 - t) a + t b is off
// by at most ~2 ulps of max(|a|, |b|) per coordinate, so a vertex comes that
// close to an endpoint only if t * h <= 2^-22 * max|coord| (h the spacing);
// tau = 2^-20 * (1 + max|coord| / h) keeps a factor of 4 on that, and the same
// holds for 1 - t.
float snap_tau_box(int nx, int ny, int nz, const float* amin_, const float* asize) {
    const int n[3] = {nx, ny, nz};
    double r = 0;
    for (int k = 0; k < 3; ++k) {
        const double amin = amin_[k], amax = double(amin_[k]) + double(asize[k]);
        const double size = asize[k];
        const double m = std::max(std::fabs(amin), std::fabs(amax));
        if (size == 0.0 || !std::isfinite(size)) return 1.0f;
        r = std::max(r, m * double(std::max(n[k] - 1, 1)) / std::fabs(size));
    }
    const double tau = std::ldexp(1.0, -20) * (1.0 + r);
    return tau >= 0.5 ? 1.0f : float(tau);
}

float snap_tau(const McParams& p) { return snap_tau_box(p.nx, p.ny, p.nz, p.amin, p.asize); }

size_t mc_workspace_bytes(int nx, int ny, int nz, long long capV, long long capF) {
    return carve(nx, ny, nz, capV, capF, nullptr).total;
}

int mc_launch(const McParams& p, void* ws, size_t ws_bytes, cudaStream_t st) {
    const McWs w0 = carve(p.nx, p.ny, p.nz, p.capV, p.capF, nullptr);
    if (ws_bytes < w0.total) return iso::fail_code(ISO_ERR_WORKSPACE);
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    const McWs w = carve(p.nx, p.ny, p.nz, p.capV, p.capF, base);
    McGrid g;
    g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
    g.NW = (p.nz + 31) / 32;
    g.dNW = make_fastdiv(uint32_t(g.NW));
    g.dNY = make_fastdiv(uint32_t(g.ny));
    g.PW = (long long)p.nx * p.ny * g.NW;
    g.level = p.level;
    g.method = p.method;
    g.tau = snap_tau(p);
    g.fma = iso::arith_fma();
    g.lgseg = iso::tune_get(iso::TUNE_MC_COUNT_THREADS) == 128 ? 9 : 10;
    g.gc = w.gc;
    if (g.PW > 0xffffffffll) return iso::fail_code(ISO_ERR_ARG);
    {
        iso::ProfScope ps("mc_signs", st);
        mc_signs_launch(p.vals, p.nx, p.ny, p.nz, p.level, w.S, st, w.ctr, (long long)(zeroed_bytes(w.nBlk) / 8));
        if (cudaGetLastError() != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    }
    const int rc = launch_count_emit(p, g, w, st);
    if (rc) return rc;
    return 0;
}

// Test hook of the bounded waits (no counterpart in isoext): runs the scan's
// look-back for chunk 32 over `state` (device, >= 32 zeroed u64, never
// published) with a limit of spin_limit polls; *status (device) becomes
// ISO_ERR_TIMEOUT and the kernel returns.  spin_limit <= 2^20.
extern "C" int iso_test_wait_timeout(unsigned spin_limit, unsigned long long* state, int* status,
                                     unsigned long long* out, void* stream) {
    if (!state || !status || !out || spin_limit > (1u << 20)) return iso::fail_code(ISO_ERR_ARG);
    lookback_probe<<<1, 32, 0, reinterpret_cast<cudaStream_t>(stream)>>>(state, 32u, spin_limit, status, out);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}
