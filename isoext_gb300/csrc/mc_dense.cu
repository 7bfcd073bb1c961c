// Dense-grid marching cubes on sm_103a.
//
// Five launches on one stream, nothing read back by the host:
//   1. mc_signs   streams the grid once (one warp per row, 16 coalesced
//                 128-byte loads in flight per warp) into a sign bitmap,
//                 1 bit per point.  This is the only pass over all values.
//   2. mc_count   one thread per point word, from the bitmap alone (16.8 MB at
//                 512^3, L2-resident): crossed-edge masks along x, y and z, active
//                 cells, face counts from the case tables; block-local vertex
//                 offsets per word; words with vertices or faces are appended to
//                 a list (one atomic per warp).
//   3. mc_scan    exclusive prefix of the per-block (V, F) sums; capacity check.
//   4. mc_emit    one thread per listed word: vertex positions at their slots
//                 (values are read only at crossed edges), faces at the word's
//                 face offset with vertex indices by rank.
//   5. mc_fixup   cooperative; returns at once unless some vertex rounded exactly
//                 onto a grid point ("snapped").  Then it merges snapped vertices
//                 by exact position, drops faces that became degenerate and
//                 compacts vertices and faces, keeping their order.
//
// Equivalence with the reference (src/mc/mc.cu:17-68): the reference emits the
// triangles of active cells in ascending cell id, drops triangles with two equal
// vertex positions (src/mc/nagae.cu:71), and welds vertices by exact position
// (src/utils.cu:32-59).  Positions here use the reference's operation order
// with every FP32 operation rounded on its own, so they are bit-identical.  Two
// distinct crossed edges give equal positions only when both vertices land on
// the same grid point (on grids whose spacing is far above float resolution;
// the host layer handles the rest), and those are the snapped vertices the
// fix-up merges.  Every crossed edge of a cell appears in its triangles (both
// tables), so without snaps the vertex set is exactly the crossed edges.
// Vertices come in edge order (the reference sorts them by position; the mesh
// is the same after relabelling).
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "mc_dense.cuh"
#include "profile.cuh"

namespace {

// ---------------------------------------------------------------------------
// Geometry shared by the kernels.

struct McGrid {
    int nx, ny, nz, NW;
    long long PW;     // point words nx * ny * NW
    float level;
    int method;
    const float* gc;  // grid coordinates: x [nx], then y [ny], then z [nz]
};

// Workspace carved from one buffer (offsets 256-aligned).
struct McWs {
    uint32_t* S;                // sign bitmap [PW]
    uint32_t* info;             // per word: segment-local vertex offset | popc(ex) << 17 | popc(ey) << 23
    unsigned long long* blk;    // per segment of words: (V, F) sums, then exclusive offsets
    uint2* list;                // words with output: (pw, segment-local face offset)
    unsigned long long* ctr;    // [0] list size [1] snaps [2] barrier count [3] barrier gen [4] V' [5] F'
    float* gc;                  // grid coordinates [nx + ny + nz] (x, then y, then z)
    uint32_t* snaps;            // snapped vertex slots [capV]
    uint32_t* table;            // position hash of snapped vertices [HC]
    uint32_t* used;             // vertex used bits [capV / 32 + 1]
    uint32_t* newidx;           // compacted vertex index [capV]
    unsigned long long* chunkF; // per chunk of faces: kept count -> offset
    unsigned long long* chunkV; // per chunk of vertices: used count -> offset
    int32_t* ftmp;              // compacted faces [capF, 3]
    float* vtmp;                // compacted vertices [capV, 3]
    long long nBlk;             // segments of SEG point words
    long long nChunkF, nChunkV;
    uint32_t HC;
    size_t total;
};

constexpr int FIX_BLOCK = 512;
constexpr int CNT_THREADS = 256;             // count kernel CTA size
constexpr int WPT = 4;                       // point words per count thread
constexpr uint32_t SEG = CNT_THREADS * WPT;  // words per segment (one scan entry)

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

uint32_t hash_cap(long long capV) {
    uint32_t c = 1024;
    while ((long long)c < 2 * capV + 1024) c <<= 1;
    return c;
}

McWs carve(int nx, int ny, int nz, long long capV, long long capF, uint8_t* base) {
    McWs w{};
    const long long NW = (nz + 31) / 32;
    const long long PW = (long long)nx * ny * NW;
    w.nBlk = (PW + SEG - 1) / SEG;
    w.nChunkF = (capF + FIX_BLOCK - 1) / FIX_BLOCK + 1;
    w.nChunkV = (capV + FIX_BLOCK - 1) / FIX_BLOCK + 1;
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
    w.list = reinterpret_cast<uint2*>(take(size_t(PW) * 8));
    w.ctr = reinterpret_cast<unsigned long long*>(take(8 * 8));
    w.gc = reinterpret_cast<float*>(take(size_t(nx + ny + nz) * 4));
    w.snaps = reinterpret_cast<uint32_t*>(take(size_t(capV) * 4));
    w.table = reinterpret_cast<uint32_t*>(take(size_t(w.HC) * 4));
    w.used = reinterpret_cast<uint32_t*>(take(size_t(capV / 32 + 1) * 4));
    w.newidx = reinterpret_cast<uint32_t*>(take(size_t(capV) * 4));
    w.chunkF = reinterpret_cast<unsigned long long*>(take(size_t(w.nChunkF) * 8));
    w.chunkV = reinterpret_cast<unsigned long long*>(take(size_t(w.nChunkV) * 8));
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

__device__ __forceinline__ const signed char* tri_row(int method, uint32_t cs) {
    return method == 0 ? ISO_TRI_NAGAE + cs * 15 : ISO_TRI_LORENSEN + cs * 12;
}

// Triangle count of each case, into shared memory.
__device__ __forceinline__ void load_ntri(int method, uint8_t* nt) {
    const int ml = method == 0 ? 15 : 12;
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        const signed char* tr = tri_row(method, uint32_t(c));
        int n = 0;
        while (n * 3 < ml && tr[n * 3] >= 0) ++n;
        nt[c] = uint8_t(n);
    }
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
// 2. count (persistent CTAs; a segment of SEG point words per iteration)

__device__ __forceinline__ void advance(const McGrid& g, int& x, int& y, int& w) {
    if (++w == g.NW) {
        w = 0;
        if (++y == g.ny) { y = 0; ++x; }
    }
}

__global__ void __launch_bounds__(CNT_THREADS) mc_count(const McGrid g, const float amin0, const float amin1,
                                                        const float amin2, const float size0, const float size1,
                                                        const float size2, const uint32_t* __restrict__ S,
                                                        uint32_t* __restrict__ info,
                                                        unsigned long long* __restrict__ blk,
                                                        uint2* __restrict__ list, unsigned long long* ctr,
                                                        float* __restrict__ gc, const uint32_t nseg) {
    __shared__ uint8_t nt[256];
    __shared__ uint32_t sm[64];
    for (int c = threadIdx.x; c < 256; c += CNT_THREADS) nt[c] = ISO_NTRI[g.method * 256 + c];
    // grid coordinates (include/utils.cuh:62-80), read by the emit kernel
    const uint32_t ncoord = uint32_t(g.nx + g.ny + g.nz);
    for (uint32_t i = blockIdx.x * CNT_THREADS + threadIdx.x; i < ncoord; i += gridDim.x * CNT_THREADS) {
        if (i < uint32_t(g.nx)) gc[i] = iso::grid_coord(i, g.nx, amin0, size0);
        else if (i < uint32_t(g.nx + g.ny)) gc[i] = iso::grid_coord(i - g.nx, g.ny, amin1, size1);
        else gc[i] = iso::grid_coord(i - g.nx - g.ny, g.nz, amin2, size2);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (uint32_t seg = blockIdx.x; seg < nseg; seg += gridDim.x) {
        const uint32_t pw0 = seg * SEG + threadIdx.x * WPT;
        uint32_t nv[WPT], nf[WPT], cxy[WPT];
        int x = 0, y = 0, w = 0;
        if (pw0 < g.PW) {
            const uint32_t row = pw0 / uint32_t(g.NW);
            w = int(pw0 - row * uint32_t(g.NW));
            x = int(row / uint32_t(g.ny));
            y = int(row - uint32_t(x) * uint32_t(g.ny));
        }
#pragma unroll
        for (int k = 0; k < WPT; ++k) {
            nv[k] = 0; nf[k] = 0; cxy[k] = 0;
            if (pw0 + k < g.PW) {
                Words d;
                load_words(g, S, pw0 + k, x, y, w, d);
                const uint32_t zm = zmask(g, w);
                const uint32_t ex = d.hasx ? (d.s[0][0][0] ^ d.s[1][0][0]) : 0u;
                const uint32_t ey = d.hasy ? (d.s[0][0][0] ^ d.s[0][1][0]) : 0u;
                const uint32_t ez = ez_of(d.s[0][0][0], d.s[0][0][1], zm);
                nv[k] = __popc(ex) + __popc(ey) + __popc(ez);
                cxy[k] = (uint32_t(__popc(ex)) << 17) | (uint32_t(__popc(ey)) << 23);
                uint32_t act = active_cells(d, zm);
                while (act) {
                    const int b = __ffs(act) - 1;
                    act &= act - 1;
                    nf[k] += nt[cell_case(d, b)];
                }
                advance(g, x, y, w);
            }
        }
        uint32_t sv = 0, sf = 0, nlive = 0;
#pragma unroll
        for (int k = 0; k < WPT; ++k) { sv += nv[k]; sf += nf[k]; nlive += (nv[k] | nf[k]) != 0; }
        uint32_t ev, ef, tv, tf;
        block_scan2<CNT_THREADS>(sv, sf, ev, ef, tv, tf, sm);
        // per-word entries and the list of words with output
        uint32_t lpos = nlive;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, lpos, d);
            if (lane >= d) lpos += u;
        }
        const uint32_t wtot = __shfl_sync(~0u, lpos, 31);
        unsigned long long lbase = 0;
        if (lane == 31 && wtot) lbase = atomicAdd(ctr, (unsigned long long)wtot);
        lbase = __shfl_sync(~0u, lbase, 31) + (lpos - nlive);
#pragma unroll
        for (int k = 0; k < WPT; ++k) {
            if (pw0 + k < g.PW) {
                info[pw0 + k] = ev | cxy[k];
                if (nv[k] | nf[k]) list[lbase++] = make_uint2(pw0 + k, ef);
            }
            ev += nv[k];
            ef += nf[k];
        }
        if (threadIdx.x == 0) {
            blk[2 * seg] = tv;
            blk[2 * seg + 1] = tf;
        }
    }
}


// ---------------------------------------------------------------------------
// 3. scan of block sums (one CTA; each thread scans a run of blocks serially)

constexpr int SCAN_THREADS = 1024;

__global__ void __launch_bounds__(SCAN_THREADS) mc_scan(unsigned long long* blk, long long nblk,
                                                        long long* counts, int* status, long long capV,
                                                        long long capF) {
    __shared__ unsigned long long wa[32], wb[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long per = (nblk + SCAN_THREADS - 1) / SCAN_THREADS;
    const long long b0 = min(nblk, tid * per), b1 = min(nblk, b0 + per);
    unsigned long long sa = 0, sb = 0;
    for (long long i = b0; i < b1; ++i) { sa += blk[2 * i]; sb += blk[2 * i + 1]; }
    unsigned long long ia = sa, ib = sb;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long x = __shfl_up_sync(~0u, ia, d), y = __shfl_up_sync(~0u, ib, d);
        if (lane >= d) { ia += x; ib += y; }
    }
    if (lane == 31) { wa[warp] = ia; wb[warp] = ib; }
    __syncthreads();
    if (warp == 0) {
        unsigned long long x = wa[lane], y = wb[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long u = __shfl_up_sync(~0u, x, d), v = __shfl_up_sync(~0u, y, d);
            if (lane >= d) { x += u; y += v; }
        }
        wa[lane] = x;
        wb[lane] = y;
    }
    __syncthreads();
    unsigned long long oa = (warp ? wa[warp - 1] : 0ull) + ia - sa;
    unsigned long long ob = (warp ? wb[warp - 1] : 0ull) + ib - sb;
    for (long long i = b0; i < b1; ++i) {
        const unsigned long long a = blk[2 * i], b = blk[2 * i + 1];
        blk[2 * i] = oa;
        blk[2 * i + 1] = ob;
        oa += a;
        ob += b;
    }
    if (tid == 0) {
        const unsigned long long V = wa[31], F = wb[31];
        counts[0] = (long long)V;
        counts[1] = (long long)F;
        if ((long long)V > capV || (long long)F > capF || V > 0x7fffffffull)
            atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
    }
}

// ---------------------------------------------------------------------------
// 4. emit (warp-cooperative: the set bits of 32 listed words are spread over
// the lanes, so each lane handles one vertex, then one cell, at a time)

__device__ __forceinline__ float gx(const McGrid& g, int x) { return g.gc[x]; }
__device__ __forceinline__ float gy(const McGrid& g, int y) { return g.gc[g.nx + y]; }
__device__ __forceinline__ float gz(const McGrid& g, int z) { return g.gc[g.nx + g.ny + z]; }

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

struct EmitWarp {
    uint32_t wd[8][32];   // bitmap words (dx, dy, ww) of each lane's word
    uint32_t nb[8][32];   // vertex slot base of the 8 neighbouring words
    uint16_t nc[8][32];   // popc(ex) | popc(ey) << 8 of those words
    uint8_t fo[32][32];   // face offset within the word of the cell at each bit
    uint32_t vid[12][32];
};

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) mc_emit(const McGrid g, const float* __restrict__ vals,
                                                 const uint32_t* __restrict__ S, const uint32_t* __restrict__ info,
                                                 const unsigned long long* __restrict__ blk,
                                                 const uint2* __restrict__ list, unsigned long long* ctr,
                                                 uint32_t* __restrict__ snaps, float* __restrict__ vout,
                                                 int32_t* __restrict__ fout, const long long* __restrict__ counts,
                                                 long long capV, long long capF) {
    constexpr int NWARP = BLOCK / 32;
    __shared__ signed char tri[256 * 15];
    __shared__ uint16_t est[256];
    __shared__ uint8_t nt[256];
    __shared__ EmitWarp ew[NWARP];
    const int ml = g.method == 0 ? 15 : 12;
    for (int i = threadIdx.x; i < 256 * ml; i += BLOCK) tri[i] = tri_row(g.method, 0)[i];
    for (int i = threadIdx.x; i < 256; i += BLOCK) {
        est[i] = ISO_EDGE_STATUS[i];
        nt[i] = ISO_NTRI[g.method * 256 + i];
    }
    __syncthreads();
    if (counts[0] > capV || counts[1] > capF || counts[0] > 0x7fffffffll) return;
    const uint32_t nlist = uint32_t(ctr[0]);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    EmitWarp& W = ew[warp];
    const uint32_t sxw = uint32_t(g.ny) * uint32_t(g.NW);
    const long long sxv = (long long)g.ny * g.nz;

    for (uint32_t c0 = (blockIdx.x * NWARP + warp) * 32u; c0 < nlist; c0 += gridDim.x * NWARP * 32u) {
        // this lane's word
        const uint32_t it = c0 + lane;
        const bool have = it < nlist;
        uint32_t pw = 0, fbase = 0, vbase = 0, ex = 0, ey = 0, ez = 0, act = 0;
        int x = 0, y = 0, w = 0;
        Words d{};
        if (have) {
            const uint2 e = list[it];
            pw = e.x;
            const uint32_t row = pw / uint32_t(g.NW);
            w = int(pw - row * uint32_t(g.NW));
            x = int(row / uint32_t(g.ny));
            y = int(row - uint32_t(x) * uint32_t(g.ny));
            load_words(g, S, pw, x, y, w, d);
            const uint32_t zm = zmask(g, w);
            ex = d.hasx ? (d.s[0][0][0] ^ d.s[1][0][0]) : 0u;
            ey = d.hasy ? (d.s[0][0][0] ^ d.s[0][1][0]) : 0u;
            ez = ez_of(d.s[0][0][0], d.s[0][0][1], zm);
            act = active_cells(d, zm);
            const uint32_t sg = pw / SEG;
            vbase = uint32_t(blk[2 * sg]) + (info[pw] & 0x1ffffu);
            fbase = uint32_t(blk[2 * sg + 1]) + e.y;
        }

        // vertices: slot vbase + k for the k-th set bit of (ex, ey, ez)
        {
            const uint32_t nvl = __popc(ex) + __popc(ey) + __popc(ez);
            uint32_t incl = nvl;
#pragma unroll
            for (int dd = 1; dd < 32; dd <<= 1) {
                const uint32_t u = __shfl_up_sync(~0u, incl, dd);
                if (lane >= dd) incl += u;
            }
            const uint32_t total = __shfl_sync(~0u, incl, 31);
            for (uint32_t r = 0; r < total; r += 32) {
                const uint32_t j = r + lane;
                const int o = owner_of(incl, j);
                const uint32_t oex = __shfl_sync(~0u, ex, o), oey = __shfl_sync(~0u, ey, o),
                               oez = __shfl_sync(~0u, ez, o);
                const uint32_t oexcl = __shfl_sync(~0u, incl - nvl, o);
                const uint32_t ovb = __shfl_sync(~0u, vbase, o);
                const int ox = __shfl_sync(~0u, x, o), oy = __shfl_sync(~0u, y, o), ow = __shfl_sync(~0u, w, o);
                if (j >= total) continue;
                const int k = int(j - oexcl);
                const int cx = __popc(oex), cy = __popc(oey);
                int ax, b;
                if (k < cx) { ax = 0; b = nth_set(oex, k); }
                else if (k < cx + cy) { ax = 1; b = nth_set(oey, k - cx); }
                else { ax = 2; b = nth_set(oez, k - cx - cy); }
                const int z = 32 * ow + b;
                const long long ia = ((long long)ox * g.ny + oy) * g.nz + z;
                const long long step = ax == 0 ? sxv : (ax == 1 ? (long long)g.nz : 1ll);
                const float va = __ldg(vals + ia), vb = __ldg(vals + ia + step);
                const float t = iso::cross_t(g.level, va, vb);
                const float xa = gx(g, ox), ya = gy(g, oy), za = gz(g, z);
                const float xb = ax == 0 ? gx(g, ox + 1) : xa;
                const float yb = ax == 1 ? gy(g, oy + 1) : ya;
                const float zb = ax == 2 ? gz(g, z + 1) : za;
                const float px = iso::lerp1(t, xa, xb), py = iso::lerp1(t, ya, yb), pz = iso::lerp1(t, za, zb);
                const uint32_t vi = ovb + uint32_t(k);
                float* vo = vout + 3ll * vi;
                vo[0] = px;
                vo[1] = py;
                vo[2] = pz;
                if ((px == xa && py == ya && pz == za) || (px == xb && py == yb && pz == zb)) {
                    const unsigned long long sidx = atomicAdd(ctr + 1, 1ull);
                    if ((long long)sidx < capV) snaps[sidx] = vi;
                }
            }
        }

        // per-word tables for the faces: words, neighbour slot bases, face offsets
        if (act) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int dx = q >> 2, dy = (q >> 1) & 1, ww = q & 1;
                W.wd[q][lane] = d.s[dx][dy][ww];
                uint32_t bse = 0, cc = 0;
                if (ww == 0 || w + 1 < g.NW) {
                    const uint32_t qw = pw + uint32_t(dx) * sxw + uint32_t(dy) * uint32_t(g.NW) + uint32_t(ww);
                    const uint32_t inf = info[qw];
                    bse = uint32_t(blk[2 * (qw / SEG)]) + (inf & 0x1ffffu);
                    cc = ((inf >> 17) & 63u) | (((inf >> 23) & 63u) << 8);
                }
                W.nb[q][lane] = bse;
                W.nc[q][lane] = uint16_t(cc);
            }
            uint32_t m = act, run = 0;
            while (m) {
                const int b = __ffs(m) - 1;
                m &= m - 1;
                W.fo[lane][b] = uint8_t(run);
                run += nt[cell_case(d, b)];
            }
        }
        __syncwarp();

        // faces: one active cell per lane
        {
            const uint32_t na = __popc(act);
            uint32_t incl = na;
#pragma unroll
            for (int dd = 1; dd < 32; dd <<= 1) {
                const uint32_t u = __shfl_up_sync(~0u, incl, dd);
                if (lane >= dd) incl += u;
            }
            const uint32_t total = __shfl_sync(~0u, incl, 31);
            for (uint32_t r = 0; r < total; r += 32) {
                const uint32_t j = r + lane;
                const int o = owner_of(incl, j);
                const uint32_t oact = __shfl_sync(~0u, act, o);
                const uint32_t oexcl = __shfl_sync(~0u, incl - na, o);
                const uint32_t ofb = __shfl_sync(~0u, fbase, o);
                const int ow = __shfl_sync(~0u, w, o);
                if (j >= total) continue;
                const int b = nth_set(oact, int(j - oexcl));
                Words c;
#pragma unroll
                for (int q = 0; q < 8; ++q) c.s[q >> 2][(q >> 1) & 1][q & 1] = W.wd[q][o];
                const uint32_t zm = zmask(g, ow);
                const uint32_t cs = cell_case(c, b);
                const uint32_t es = est[cs];
#pragma unroll
                for (int k = 0; k < 12; ++k) {
                    if (!((es >> k) & 1u)) continue;
                    const int a = iso_edge_corner(2 * k), cc = iso_edge_corner(2 * k + 1);
                    const int ax = (cc - a) == 4 ? 0 : ((cc - a) == 2 ? 1 : 2);
                    const int adx = a >> 2, ady = (a >> 1) & 1, adz = a & 1;
                    const int ww = adz ? ((b + 1) >> 5) : 0;
                    const int bit = (b + adz) & 31;
                    const int q0 = (adx * 2 + ady) * 2;  // neighbour word index with ww = 0
                    uint32_t mm, off = ww ? W.nb[q0 + 1][o] : W.nb[q0][o];
                    const uint32_t cxy = ww ? W.nc[q0 + 1][o] : W.nc[q0][o];
                    if (ax == 0) {
                        mm = ww ? (c.s[0][ady][1] ^ c.s[1][ady][1]) : (c.s[0][ady][0] ^ c.s[1][ady][0]);
                    } else if (ax == 1) {
                        mm = ww ? (c.s[adx][0][1] ^ c.s[adx][1][1]) : (c.s[adx][0][0] ^ c.s[adx][1][0]);
                        off += cxy & 0xffu;
                    } else {
                        mm = ez_of(c.s[adx][ady][0], c.s[adx][ady][1], zm);
                        off += (cxy & 0xffu) + (cxy >> 8);
                    }
                    W.vid[k][lane] = off + __popc(mm & ((1u << bit) - 1u));
                }
                unsigned long long fo = (unsigned long long)ofb + W.fo[o][b];
                const signed char* tr = tri + cs * ml;
                for (int k = 0; k < ml && tr[k] >= 0; k += 3) {
                    int32_t* f3 = fout + 3 * fo;
                    f3[0] = int32_t(W.vid[tr[k]][lane]);
                    f3[1] = int32_t(W.vid[tr[k + 1]][lane]);
                    f3[2] = int32_t(W.vid[tr[k + 2]][lane]);
                    ++fo;
                }
            }
        }
        __syncwarp();
    }
}


// ---------------------------------------------------------------------------
// 5. snap fix-up (cooperative launch: all CTAs are resident)

struct FixArgs {
    float* vout;
    int32_t* fout;
    long long* counts;
    int* status;
    long long capV, capF;
    McWs w;
};

// Grid-wide barrier with a bounded wait; false if it ran out (status set).
__device__ bool grid_barrier(unsigned long long* ctr, int* status) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned long long* gen = ctr + 3;
        const unsigned long long g0 = *gen;
        __threadfence();
        const unsigned long long arrived = atomicAdd(ctr + 2, 1ull);
        if (arrived == gridDim.x - 1) {
            ctr[2] = 0;
            __threadfence();
            atomicAdd(ctr + 3, 1ull);
        } else {
            uint32_t spins = 0;
            while (*gen == g0) {
                if (++spins > ISO_SPIN_LIMIT) {
                    atomicCAS(status, 0, int(ISO_ERR_TIMEOUT));
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ uint32_t pbits(float f) { return __float_as_uint(f == 0.0f ? 0.0f : f); }
__device__ __forceinline__ uint32_t phash(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}

// Vertex with the smallest index at vertex v's position among snapped vertices, or v.
__device__ uint32_t rep_of(const FixArgs& a, uint32_t v) {
    const float* p = a.vout + 3ll * v;
    const uint32_t k0 = pbits(p[0]), k1 = pbits(p[1]), k2 = pbits(p[2]);
    const uint32_t mask = a.w.HC - 1;
    uint32_t h = phash(k0, k1, k2) & mask;
    for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const uint32_t j = a.w.table[h];
        if (j == 0xffffffffu) break;
        const float* q = a.vout + 3ll * j;
        if (pbits(q[0]) == k0 && pbits(q[1]) == k1 && pbits(q[2]) == k2) return j;
    }
    return v;
}

__device__ __forceinline__ uint32_t block_excl(uint32_t x, uint32_t& total, uint32_t* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t u = __shfl_up_sync(~0u, inc, d);
        if (lane >= d) inc += u;
    }
    if (lane == 31) sm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t y = lane < FIX_BLOCK / 32 ? sm[lane] : 0u;
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

// Exclusive scan of n counts in place (one CTA), returns the total.
__device__ unsigned long long scan_serial(unsigned long long* c, long long n, unsigned long long* sm64) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long per = (n + FIX_BLOCK - 1) / FIX_BLOCK;
    const long long i0 = min(n, tid * per), i1 = min(n, i0 + per);
    unsigned long long s = 0;
    for (long long i = i0; i < i1; ++i) s += c[i];
    unsigned long long inc = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long u = __shfl_up_sync(~0u, inc, d);
        if (lane >= d) inc += u;
    }
    if (lane == 31) sm64[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned long long y = lane < FIX_BLOCK / 32 ? sm64[lane] : 0ull;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long u = __shfl_up_sync(~0u, y, d);
            if (lane >= d) y += u;
        }
        sm64[lane] = y;
    }
    __syncthreads();
    unsigned long long o = (warp ? sm64[warp - 1] : 0ull) + inc - s;
    for (long long i = i0; i < i1; ++i) {
        const unsigned long long v = c[i];
        c[i] = o;
        o += v;
    }
    const unsigned long long total = sm64[31];
    __syncthreads();
    return total;
}

__device__ __forceinline__ bool face_keep(const int32_t* f) {
    return f[0] != f[1] && f[0] != f[2] && f[1] != f[2];
}

__global__ void __launch_bounds__(FIX_BLOCK) mc_fixup(const FixArgs a) {
    __shared__ uint32_t sm[32];
    __shared__ unsigned long long sm64[32];
    const McWs& w = a.w;
    const long long V = a.counts[0], F = a.counts[1];
    if (V > a.capV || F > a.capF || V > 0x7fffffffll) return;
    const long long nsnap = min((long long)w.ctr[1], a.capV);
    if (nsnap == 0) return;
    const long long gtid = (long long)blockIdx.x * FIX_BLOCK + threadIdx.x;
    const long long gstride = (long long)gridDim.x * FIX_BLOCK;
    const uint32_t mask = w.HC - 1;

    for (long long i = gtid; i < w.HC; i += gstride) w.table[i] = 0xffffffffu;
    for (long long i = gtid; i < V / 32 + 1; i += gstride) w.used[i] = 0u;
    if (!grid_barrier(w.ctr, a.status)) return;

    // snapped vertices into the position hash; smallest index wins
    for (long long s = gtid; s < nsnap; s += gstride) {
        const uint32_t v = w.snaps[s];
        const float* p = a.vout + 3ll * v;
        const uint32_t k0 = pbits(p[0]), k1 = pbits(p[1]), k2 = pbits(p[2]);
        uint32_t h = phash(k0, k1, k2) & mask;
        bool done = false;
        for (uint32_t probe = 0; probe <= mask && !done; ++probe, h = (h + 1) & mask) {
            const uint32_t cur = atomicCAS(&w.table[h], 0xffffffffu, v);
            if (cur == 0xffffffffu) { done = true; break; }
            const float* q = a.vout + 3ll * cur;
            if (pbits(q[0]) == k0 && pbits(q[1]) == k1 && pbits(q[2]) == k2) {
                atomicMin(&w.table[h], v);
                done = true;
            }
        }
        if (!done) atomicCAS(a.status, 0, int(ISO_ERR_OVERFLOW));
    }
    if (!grid_barrier(w.ctr, a.status)) return;

    // faces: merge snapped vertices, count the non-degenerate ones per chunk
    const long long nchF = (F + FIX_BLOCK - 1) / FIX_BLOCK;
    for (long long c = blockIdx.x; c < nchF; c += gridDim.x) {
        const long long f = c * FIX_BLOCK + threadIdx.x;
        uint32_t keep = 0;
        if (f < F) {
            int32_t* fp = a.fout + 3 * f;
#pragma unroll
            for (int k = 0; k < 3; ++k) fp[k] = int32_t(rep_of(a, uint32_t(fp[k])));
            keep = face_keep(fp);
        }
        uint32_t tot;
        block_excl(keep, tot, sm);
        if (threadIdx.x == 0) w.chunkF[c] = tot;
    }
    if (!grid_barrier(w.ctr, a.status)) return;
    if (blockIdx.x == 0) {
        const unsigned long long Fn = scan_serial(w.chunkF, nchF, sm64);
        if (threadIdx.x == 0) w.ctr[5] = Fn;
    }
    if (!grid_barrier(w.ctr, a.status)) return;

    // kept faces, in order, to ftmp; mark the vertices they use
    for (long long c = blockIdx.x; c < nchF; c += gridDim.x) {
        const long long f = c * FIX_BLOCK + threadIdx.x;
        uint32_t keep = 0;
        const int32_t* fp = a.fout + 3 * (f < F ? f : 0);
        if (f < F) keep = face_keep(fp);
        uint32_t tot;
        const uint32_t ex = block_excl(keep, tot, sm);
        if (keep) {
            int32_t* o = w.ftmp + 3 * (w.chunkF[c] + ex);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                o[k] = fp[k];
                atomicOr(&w.used[uint32_t(fp[k]) >> 5], 1u << (uint32_t(fp[k]) & 31u));
            }
        }
    }
    if (!grid_barrier(w.ctr, a.status)) return;

    // used vertices per chunk
    const long long nchV = (V + FIX_BLOCK - 1) / FIX_BLOCK;
    for (long long c = blockIdx.x; c < nchV; c += gridDim.x) {
        const long long v = c * FIX_BLOCK + threadIdx.x;
        const uint32_t u = v < V ? (w.used[v >> 5] >> (v & 31)) & 1u : 0u;
        uint32_t tot;
        block_excl(u, tot, sm);
        if (threadIdx.x == 0) w.chunkV[c] = tot;
    }
    if (!grid_barrier(w.ctr, a.status)) return;
    if (blockIdx.x == 0) {
        const unsigned long long Vn = scan_serial(w.chunkV, nchV, sm64);
        if (threadIdx.x == 0) w.ctr[4] = Vn;
    }
    if (!grid_barrier(w.ctr, a.status)) return;

    // compacted vertices to vtmp, new indices
    for (long long c = blockIdx.x; c < nchV; c += gridDim.x) {
        const long long v = c * FIX_BLOCK + threadIdx.x;
        const uint32_t u = v < V ? (w.used[v >> 5] >> (v & 31)) & 1u : 0u;
        uint32_t tot;
        const uint32_t ex = block_excl(u, tot, sm);
        if (u) {
            const unsigned long long j = w.chunkV[c] + ex;
            w.newidx[v] = uint32_t(j);
            w.vtmp[3 * j] = a.vout[3 * v];
            w.vtmp[3 * j + 1] = a.vout[3 * v + 1];
            w.vtmp[3 * j + 2] = a.vout[3 * v + 2];
        }
    }
    if (!grid_barrier(w.ctr, a.status)) return;

    const long long Vn = (long long)w.ctr[4], Fn = (long long)w.ctr[5];
    for (long long j = gtid; j < 3 * Vn; j += gstride) a.vout[j] = w.vtmp[j];
    for (long long j = gtid; j < 3 * Fn; j += gstride) a.fout[j] = int32_t(w.newidx[w.ftmp[j]]);
    if (gtid == 0) {
        a.counts[0] = Vn;
        a.counts[1] = Fn;
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
                                                       int nz, float level, uint32_t* __restrict__ out) {
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
                    v[u] = (w0 + u < NWg && z < nz) ? __ldg(rp + z) : level;
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

template <int BLOCK>
int launch_count_emit(const McParams& p, const McGrid& g, const McWs& w, cudaStream_t st) {
    const int sms = sm_count();
    {
        iso::ProfScope ps("mc_count", st);
        static int per = -1;
        if (per < 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mc_count, CNT_THREADS, 0);
        const long long grid = std::max<long long>(1, std::min<long long>(w.nBlk, (long long)sms * std::max(per, 1)));
        mc_count<<<unsigned(grid), CNT_THREADS, 0, st>>>(g, p.amin[0], p.amin[1], p.amin[2], p.asize[0], p.asize[1],
                                                         p.asize[2], w.S, w.info, w.blk, w.list, w.ctr, w.gc,
                                                         uint32_t(w.nBlk));
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    {
        iso::ProfScope ps("mc_scan", st);
        mc_scan<<<1, SCAN_THREADS, 0, st>>>(w.blk, w.nBlk, p.counts, p.status, p.capV, p.capF);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    {
        iso::ProfScope ps("mc_emit", st);
        static int per = -1;
        if (per < 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mc_emit<BLOCK>, BLOCK, 0);
        // enough warps for every listed word to have a lane, up to the resident limit
        const long long want = (w.nBlk * SEG / 32 + (BLOCK / 32) - 1) / (BLOCK / 32);
        const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sms * std::max(per, 1)));
        mc_emit<BLOCK><<<unsigned(grid), BLOCK, 0, st>>>(g, p.vals, w.S, w.info, w.blk, w.list, w.ctr, w.snaps,
                                                         p.vout, p.fout, p.counts, p.capV, p.capF);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    return 0;
}

}  // namespace

int mc_set_block(int threads) {
    if (threads != 128 && threads != 256) return ISO_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    g_block = threads;
    return 0;
}

int mc_get_block() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_block;
}

void mc_signs_launch(const float* vals, int nx, int ny, int nz, float level, uint32_t* out,
                     cudaStream_t st) {
    const long long rows = (long long)nx * ny;
    const long long want = (rows + (SIGN_BLOCK / 32) - 1) / (SIGN_BLOCK / 32);
    const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sm_count() * 32));
    mc_signs<<<unsigned(grid), SIGN_BLOCK, 0, st>>>(vals, rows, nz, level, out);
}

size_t mc_workspace_bytes(int nx, int ny, int nz, long long capV, long long capF) {
    return carve(nx, ny, nz, capV, capF, nullptr).total;
}

int mc_launch(const McParams& p, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int block = mc_get_block();
    const McWs w0 = carve(p.nx, p.ny, p.nz, p.capV, p.capF, nullptr);
    if (ws_bytes < w0.total) return ISO_ERR_WORKSPACE;
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    const McWs w = carve(p.nx, p.ny, p.nz, p.capV, p.capF, base);
    McGrid g;
    g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
    g.NW = (p.nz + 31) / 32;
    g.PW = (long long)p.nx * p.ny * g.NW;
    g.level = p.level;
    g.method = p.method;
    g.gc = w.gc;
    if (g.PW > 0xffffffffll) return ISO_ERR_ARG;
    if (cudaMemsetAsync(w.ctr, 0, 8 * 8, st) != cudaSuccess) return ISO_ERR_CUDA;
    {
        iso::ProfScope ps("mc_signs", st);
        mc_signs_launch(p.vals, p.nx, p.ny, p.nz, p.level, w.S, st);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    const int rc = block == 128 ? launch_count_emit<128>(p, g, w, st) : launch_count_emit<256>(p, g, w, st);
    if (rc) return rc;
    {
        iso::ProfScope ps("mc_fixup", st);
        static int per = -1;  // co-resident fix-up CTAs per SM
        if (per < 0) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mc_fixup, FIX_BLOCK, 0);
            per = std::max(1, std::min(n, 2));
        }
        FixArgs fa{p.vout, p.fout, p.counts, p.status, p.capV, p.capF, w};
        void* args[] = {&fa};
        const unsigned grid = unsigned(sm_count() * per);
        if (cudaLaunchCooperativeKernel((void*)mc_fixup, dim3(grid), dim3(FIX_BLOCK), args, 0, st) !=
            cudaSuccess)
            return ISO_ERR_CUDA;
    }
    return 0;
}
