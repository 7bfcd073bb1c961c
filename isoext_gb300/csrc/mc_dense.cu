// Dense-grid marching cubes on sm_103a.
//
// Four launches on one stream:
//   1. mc_signs    streams the grid once (one warp per row, 16 coalesced
//                  128-byte loads in flight per warp) into a sign bitmap,
//                  1 bit per point.
//   2. mc_extract  persistent CTAs; each work item is a column of tiles
//                  (row group, z chunk) swept along x over a chunk of planes.
//                  A ring of three planes of bitmaps (signs, crossed edges,
//                  "snap" edges whose vertex rounds exactly onto a grid point)
//                  lives in shared memory; grid values are read only for the
//                  crossed edges (lerp).  Per tile: cell activity by word-wide
//                  bit logic, face counts, vertex existence, a warp scan that
//                  takes space from per-CTA staging blocks, and staged vertices
//                  (position + key) and faces (key references).
//   3. mc_tile_scan  exclusive prefix of per-tile vertex / face counts.
//   4. mc_resolve  copies staged vertices to their final slots and turns face
//                  key references into vertex indices (one warp per tile).
//
// Equivalence with the reference (src/mc/mc.cu:17-68): the reference emits the
// triangles of active cells in ascending cell id, drops triangles with two equal
// vertex positions (src/mc/nagae.cu:71), and welds vertices by exact position
// (src/utils.cu:32-59).  Here a vertex is identified by its key -- the grid edge
// it lies on, or the grid point its lerp rounds onto exactly -- and positions are
// computed with the reference's operation order, so equal keys are equal
// positions.  Faces are written in the reference's order; vertices in ascending
// key order (the reference sorts them by position instead; same mesh after
// relabelling).
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "mc_dense.cuh"
#include "profile.cuh"

namespace {

constexpr int NB = 7;  // bitmaps kept per plane
enum { B_SGN = 0, B_LOX, B_LOY, B_LOZ, B_HIX, B_HIY, B_HIZ };
constexpr int RING = 3;  // planes P-1, P, P+1

struct Layout {
    size_t bm, cr, act, fre, snp, du, ex, vcnt, fcnt, tbl, rowoff, gx, gy, gz, zval, ecol, ocol, ocell,
        scratch, estat, tri, ntri, misc, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline Layout make_layout(const McTiles& t) {
    Layout L;
    size_t o = 0;
    const size_t rw = size_t(t.RY) * t.NW;  // words per bitmap
    L.bm = o;      o = al16(o + size_t(RING) * NB * rw * 4);
    L.cr = o;      o = al16(o + 3 * rw * 4);
    L.act = o;     o = al16(o + 2 * rw * 4);
    L.fre = o;     o = al16(o + 2 * rw * 4);
    L.snp = o;     o = al16(o + 2 * rw * 4);
    L.du = o;      o = al16(o + 4 * rw * 4);
    L.ex = o;      o = al16(o + 4 * rw * 4);
    L.vcnt = o;    o = al16(o + rw * 4);
    L.fcnt = o;    o = al16(o + rw * 4);
    L.tbl = o;     o = al16(o + 3 * rw * 4);
    L.rowoff = o;  o = al16(o + size_t(t.RY) * 8);
    L.gx = o;      o = al16(o + RING * 4);
    L.gy = o;      o = al16(o + size_t(t.RY) * 4);
    L.gz = o;      o = al16(o + size_t(32) * t.NW * 4);
    L.zval = o;    o = al16(o + size_t(t.NW) * 4);
    L.ecol = o;    o = al16(o + size_t(t.NW) * 4);
    L.ocol = o;    o = al16(o + size_t(t.NW) * 4);
    L.ocell = o;   o = al16(o + size_t(t.NW) * 4);
    L.scratch = o; o = al16(o + size_t(t.threads / 32) * 64 * 4);
    L.estat = o;   o = al16(o + 256 * 2);
    L.tri = o;     o = al16(o + 256 * 15);
    L.ntri = o;    o = al16(o + 256);
    L.misc = o;    o = al16(o + 128);
    L.total = o;
    return L;
}

using iso::next1;
using iso::prev1;

// Per-CTA state: shared-memory arrays and the current item / tile.
struct Ctx {
    // shared memory
    uint32_t* bm;
    uint32_t *cr, *act, *fre, *snp, *du, *ex, *vcnt, *fcnt, *tbl;
    long long* rowoff;
    float *gx, *gy, *gz;
    uint32_t *zval, *ecol, *ocol, *ocell;
    uint16_t* estat;
    int8_t* tri;
    uint8_t* ntri;
    unsigned long long* misc;
    // grid
    const float* vals;
    int nx, ny, nz;
    float level;
    // tiling
    int R, ZC, RY, NW, RW, nRT, nZT;
    // current item / tile
    int rt, zt, Y0, Y1, Z0, Z1;
    int P, sA, sB, sC;  // ring slots of planes P-1, P, P+1 (-1 when absent)

    __device__ __forceinline__ uint32_t* plane(int slot, int arr) const {
        return bm + (size_t(slot) * NB + arr) * RW;
    }
    __device__ __forceinline__ uint32_t bit(int slot, int arr, int row, int col) const {
        return (plane(slot, arr)[row * NW + (col >> 5)] >> (col & 31)) & 1u;
    }
    // grid value at (plane, row, col) of the current item (row/col in slab units)
    __device__ __forceinline__ float value(int pl, int row, int col) const {
        long long y = Y0 - 1 + row, z = Z0 - 32 + col;
        return __ldg(vals + ((long long)pl * ny + y) * nz + z);
    }
    __device__ __forceinline__ int slot_of(int rel) const {
        return rel == 0 ? sA : (rel == 1 ? sB : sC);
    }
};

// Case number of the cell whose highest corner is (hy, hc) in layer L.
// Corner k = 4dx + 2dy + dz is plane rel = L + dx, row hy - 1 + dy, col hc - 1 + dz.
__device__ __forceinline__ uint32_t cell_case(const Ctx& c, int L, int hy, int hc) {
    const int lo = L ? c.sB : c.sA, hi = L ? c.sC : c.sB;
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        cs |= c.bit((k >> 2) ? hi : lo, B_SGN, hy - 1 + ((k >> 1) & 1), hc - 1 + (k & 1)) << k;
    return cs;
}

// Vertex identity of each crossed edge of a cell, as corner * 4 + type
// (type 0/1/2 = edge along x/y/z keyed by its high corner, 3 = the grid point
// the edge vertex rounds onto).  Two edges of one cell share a vertex exactly
// when their codes are equal.
__device__ __forceinline__ void cell_codes(const Ctx& c, int L, int hy, int hc, uint32_t est,
                                           bool snap, uint8_t* ck) {
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        if (!((est >> e) & 1u)) continue;
        const int a = ISO_EDGE_CORNERS[2 * e], b = ISO_EDGE_CORNERS[2 * e + 1];
        const int d = b - a;
        const int ax = d == 4 ? 0 : (d == 2 ? 1 : 2);
        uint8_t code = uint8_t(b * 4 + ax);
        if (snap) {
            const int slot = c.slot_of(L + (b >> 2));
            const int row = hy - 1 + ((b >> 1) & 1), col = hc - 1 + (b & 1);
            if (c.bit(slot, B_LOX + ax, row, col)) code = uint8_t(a * 4 + 3);
            else if (c.bit(slot, B_HIX + ax, row, col)) code = uint8_t(b * 4 + 3);
        }
        ck[e] = code;
    }
}

// Number of faces a cell emits: its table count, or for a cell with snapped
// edges the triangles whose three vertices are distinct.
__device__ __forceinline__ uint32_t cell_nfaces(const Ctx& c, int L, int hy, int hc, bool snap) {
    const uint32_t cs = cell_case(c, L, hy, hc);
    if (!snap) return c.ntri[cs];
    uint8_t ck[12];
    cell_codes(c, L, hy, hc, c.estat[cs], true, ck);
    const int8_t* tr = c.tri + cs * 15;
    uint32_t nt = 0;
    for (int k = 0; k < 15 && tr[k] >= 0; k += 3) {
        const uint8_t k0 = ck[tr[k]], k1 = ck[tr[k + 1]], k2 = ck[tr[k + 2]];
        nt += (k0 != k1 && k0 != k2 && k1 != k2);
    }
    return nt;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) mc_extract(const McParams p) {
    extern __shared__ __align__(16) uint8_t smem[];
    const McTiles& T = p.t;
    const Layout LY = make_layout(T);
    Ctx c;
    c.bm = reinterpret_cast<uint32_t*>(smem + LY.bm);
    c.cr = reinterpret_cast<uint32_t*>(smem + LY.cr);
    c.act = reinterpret_cast<uint32_t*>(smem + LY.act);
    c.fre = reinterpret_cast<uint32_t*>(smem + LY.fre);
    c.snp = reinterpret_cast<uint32_t*>(smem + LY.snp);
    c.du = reinterpret_cast<uint32_t*>(smem + LY.du);
    c.ex = reinterpret_cast<uint32_t*>(smem + LY.ex);
    c.vcnt = reinterpret_cast<uint32_t*>(smem + LY.vcnt);
    c.fcnt = reinterpret_cast<uint32_t*>(smem + LY.fcnt);
    c.tbl = reinterpret_cast<uint32_t*>(smem + LY.tbl);
    c.rowoff = reinterpret_cast<long long*>(smem + LY.rowoff);
    c.gx = reinterpret_cast<float*>(smem + LY.gx);
    c.gy = reinterpret_cast<float*>(smem + LY.gy);
    c.gz = reinterpret_cast<float*>(smem + LY.gz);
    c.zval = reinterpret_cast<uint32_t*>(smem + LY.zval);
    c.ecol = reinterpret_cast<uint32_t*>(smem + LY.ecol);
    c.ocol = reinterpret_cast<uint32_t*>(smem + LY.ocol);
    c.ocell = reinterpret_cast<uint32_t*>(smem + LY.ocell);
    c.estat = reinterpret_cast<uint16_t*>(smem + LY.estat);
    c.tri = reinterpret_cast<int8_t*>(smem + LY.tri);
    c.ntri = reinterpret_cast<uint8_t*>(smem + LY.ntri);
    c.misc = reinterpret_cast<unsigned long long*>(smem + LY.misc);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARP = BLOCK / 32;
    uint32_t* wscratch = reinterpret_cast<uint32_t*>(smem + LY.scratch) + warp * 64;

    c.vals = p.vals;
    c.nx = T.nx; c.ny = T.ny; c.nz = T.nz; c.level = p.level;
    c.R = T.R; c.ZC = T.ZC; c.RY = T.RY; c.NW = T.NW; c.RW = T.RY * T.NW;
    c.nRT = T.nRT; c.nZT = T.nZT;
    const int NW = c.NW, RW = c.RW;
    const float tau = p.snapTau;

    // Lookup tables and the (layer/axis, row, word) decode table.
    for (int i = tid; i < 256; i += BLOCK) {
        c.estat[i] = ISO_EDGE_STATUS[i];
        int n = 0;
        if (p.method == 0) {
            while (n < ISO_NAGAE_MAX_TRI && ISO_TRI_NAGAE[i * 15 + 3 * n] >= 0) ++n;
        } else {
            while (n < ISO_LORENSEN_MAX_TRI && ISO_TRI_LORENSEN[i * 12 + 3 * n] >= 0) ++n;
        }
        c.ntri[i] = uint8_t(n);
    }
    for (int i = tid; i < 256 * 15; i += BLOCK) {
        int cs = i / 15, k = i % 15;
        c.tri[i] = p.method == 0 ? ISO_TRI_NAGAE[i] : (k < 12 ? ISO_TRI_LORENSEN[cs * 12 + k] : -1);
    }
    for (int i = tid; i < 3 * RW; i += BLOCK) {
        int a = i / RW, r = i - a * RW;
        int ly = r / NW, w = r - ly * NW;
        c.tbl[i] = (uint32_t(a) << 24) | (uint32_t(ly) << 16) | uint32_t(w);
    }
    if (tid < 16) c.misc[tid] = 0;  // [5..8]: current staging blocks (empty)
    __syncthreads();

    const long long perChunk = (long long)c.nRT * c.nZT;

    for (;;) {
        if (tid == 0) c.misc[0] = atomicAdd(&p.ctr[0], 1ull);
        __syncthreads();
        const long long item = (long long)c.misc[0];
        if (item >= T.nItems) break;
        const int chunk = int(item / perChunk);
        const int colidx = int(item % perChunk);
        c.rt = colidx / c.nZT;
        c.zt = colidx % c.nZT;
        c.Y0 = c.rt * c.R;
        c.Y1 = min(c.Y0 + c.R, c.ny);
        c.Z0 = c.zt * c.ZC;
        c.Z1 = min(c.Z0 + c.ZC, c.nz);
        const int Pa = chunk * T.PC, Pb = min(Pa + T.PC, c.nx);
        const int pfirst = max(Pa - 1, 0), plast = min(Pb, c.nx - 1);
        const int nslab = plast - pfirst + 1;

        // Per-item coordinates and column masks.
        const int zf = max(c.Z0 - 1, 0), zl = min(c.Z1, c.nz - 1);  // loaded z range
        const int ylo = max(c.Y0 - 1, 0), yhi = min(c.Y1, c.ny - 1);  // loaded rows
        for (int i = tid; i < 32 * NW; i += BLOCK) {
            int z = c.Z0 - 32 + i;
            c.gz[i] = (z >= 0 && z < c.nz)
                          ? iso::grid_coord(uint32_t(z), uint32_t(c.nz), p.amin[2], p.asize[2])
                          : 0.0f;
        }
        for (int i = tid; i < c.RY; i += BLOCK) {
            int y = c.Y0 - 1 + i;
            c.gy[i] = (y >= 0 && y < c.ny)
                          ? iso::grid_coord(uint32_t(y), uint32_t(c.ny), p.amin[1], p.asize[1])
                          : 0.0f;
        }
        for (int w = tid; w < NW; w += BLOCK) {
            c.zval[w] = iso::range_mask(w, zf - c.Z0 + 32, zl - c.Z0 + 32);
            // E cells by high-corner column: cz in [Z0-1, Z1-1] and in the grid
            c.ecol[w] = iso::range_mask(w, max(32, 33 - c.Z0), min(c.Z1 - 1, c.nz - 2) - c.Z0 + 33);
            // own cells: cz in [Z0-1, Z1-2]
            c.ocell[w] = iso::range_mask(w, max(32, 33 - c.Z0), c.Z1 - c.Z0 + 31);
            // owned points: z in [Z0, Z1)
            c.ocol[w] = iso::range_mask(w, 32, c.Z1 - c.Z0 + 31);
        }
        for (int i = tid; i < 4 * RW; i += BLOCK) c.du[i] = 0;
        const int hyE0 = max(1, 2 - c.Y0), hyE1 = min(c.Y1 - 1, c.ny - 2) - c.Y0 + 2;
        const int hyO0 = hyE0, hyO1 = c.Y1 - c.Y0;
        __syncthreads();

        for (int j = 0; j < nslab; ++j) {
            const int pl = pfirst + j;
            const int slot = j % RING;
            const int sp = j > 0 ? (j - 1) % RING : -1;
            if (tid == 0)
                c.gx[slot] = iso::grid_coord(uint32_t(pl), uint32_t(c.nx), p.amin[0], p.asize[0]);
            for (int i = tid; i < c.RY; i += BLOCK) {
                const int y = c.Y0 - 1 + i;
                // offset of (y, z = Z0) in the value array; -1 marks a row outside the slab
                c.rowoff[i] = (y >= ylo && y <= yhi) ? ((long long)pl * c.ny + y) * c.nz + c.Z0 : -1ll;
            }
            __syncthreads();

            // (1) sign bits of plane pl, from the bitmap mc_signs wrote: tile word w
            // covers z = Z0 - 32 + 32 w + b, i.e. bitmap word Z0 / 32 + w - 1.
            {
                uint32_t* sg = c.plane(slot, B_SGN);
                const long long NWg = (c.nz + 31) / 32;
                const long long w0 = c.Z0 / 32 - 1;
                for (int r = tid; r < RW; r += BLOCK) {
                    const uint32_t x = c.tbl[r];
                    const int ly = (x >> 16) & 0xff, w = x & 0xffff;
                    const int y = c.Y0 - 1 + ly;
                    const long long gw = w0 + w;
                    uint32_t b = 0;
                    if (c.rowoff[ly] >= 0 && gw >= 0 && gw < NWg)
                        b = __ldg(p.signs + ((long long)pl * c.ny + y) * NWg + gw) & c.zval[w];
                    sg[r] = b;
                }
            }
            __syncthreads();

            // (2) crossed edges whose high endpoint is in plane pl (word-parallel)
            for (int i = tid; i < 3 * RW; i += BLOCK) {
                const uint32_t x = c.tbl[i];
                const int ax = x >> 24, ly = (x >> 16) & 0xff, w = x & 0xffff;
                const int r = i - ax * RW;
                const bool rv = c.rowoff[ly] >= 0;
                const uint32_t* sgrow = c.plane(slot, B_SGN) + ly * NW;
                uint32_t cr = 0;
                if (rv) {
                    if (ax == 0) {
                        if (sp >= 0) cr = (sgrow[w] ^ c.plane(sp, B_SGN)[r]) & c.zval[w];
                    } else if (ax == 1) {
                        if (ly >= 1 && c.rowoff[ly - 1] >= 0) cr = (sgrow[w] ^ sgrow[w - NW]) & c.zval[w];
                    } else {
                        cr = (sgrow[w] ^ prev1(sgrow, w)) & c.zval[w] & prev1(c.zval, w);
                    }
                }
                c.cr[i] = cr;
                c.plane(slot, B_LOX + ax)[r] = 0u;
                c.plane(slot, B_HIX + ax)[r] = 0u;
            }
            __syncthreads();

            // (3) snapped edges: crossings whose vertex rounds onto an endpoint.
            // Only t within tau of 0 or 1 can round onto a grid point; those get
            // the exact test.
            iso::warp_foreach_bit(
                warp * 32, 3 * RW, NWARP * 32, wscratch, [&](int i) { return c.cr[i]; },
                [&](int i, int b) {
                    const uint32_t x = c.tbl[i];
                    const int ax = x >> 24, ly = (x >> 16) & 0xff, w = x & 0xffff;
                    const int col = 32 * w + b;
                    const int pa = ax == 0 ? pl - 1 : pl;
                    const int ra = ax == 1 ? ly - 1 : ly;
                    const int ca = ax == 2 ? col - 1 : col;
                    const float va = c.value(pa, ra, ca), vb = c.value(pl, ly, col);
                    const float t = iso::cross_t(c.level, va, vb);
                    if (t >= tau && t <= 1.0f - tau) return;  // NaN falls through
                    const float xa = c.gx[ax == 0 ? sp : slot], ya = c.gy[ra], za = c.gz[ca];
                    const float xb = c.gx[slot], yb = c.gy[ly], zb = c.gz[col];
                    const float px = iso::lerp1(t, xa, xb), py = iso::lerp1(t, ya, yb),
                                pz = iso::lerp1(t, za, zb);
                    const int r = i - ax * RW;
                    if (px == xa && py == ya && pz == za)
                        atomicOr(&c.plane(slot, B_LOX + ax)[r], 1u << b);
                    else if (px == xb && py == yb && pz == zb)
                        atomicOr(&c.plane(slot, B_HIX + ax)[r], 1u << b);
                });
            __syncthreads();

            // Tiles ready after this plane: P = pl - 1 and, at the grid's last
            // plane, P = pl itself.
            for (int pass = 0; pass < 2; ++pass) {
                const int P = pass == 0 ? pl - 1 : pl;
                if (pass == 1 && pl != c.nx - 1) break;
                if (P < Pa || P >= Pb) continue;
                c.P = P;
                c.sB = (P - pfirst) % RING;
                c.sA = P >= 1 ? (P - 1 - pfirst) % RING : -1;
                c.sC = P + 1 <= c.nx - 1 ? (P + 1 - pfirst) % RING : -1;
                const bool L0 = P >= 1, L1 = P + 1 <= c.nx - 1;

                // T1: cell masks of both layers (word-parallel); cells with
                // snapped edges mark the owned vertices their faces use.
                for (int i = tid; i < 2 * RW; i += BLOCK) {
                    const uint32_t x = c.tbl[i];
                    const int L = x >> 24, hy = (x >> 16) & 0xff, hw = x & 0xffff;
                    uint32_t act = 0, fre = 0, snp = 0;
                    const bool lok = L ? L1 : L0;
                    const uint32_t em = (lok && hy >= hyE0 && hy <= hyE1 && hw >= 1) ? c.ecol[hw] : 0u;
                    if (em) {
                        const int lo = L ? c.sB : c.sA, hi = L ? c.sC : c.sB;
                        const uint32_t* a0 = c.plane(lo, B_SGN) + (hy - 1) * NW;
                        const uint32_t* a1 = a0 + NW;
                        const uint32_t* b0 = c.plane(hi, B_SGN) + (hy - 1) * NW;
                        const uint32_t* b1 = b0 + NW;
                        const uint32_t w0 = a0[hw], w1 = prev1(a0, hw), w2 = a1[hw], w3 = prev1(a1, hw);
                        const uint32_t w4 = b0[hw], w5 = prev1(b0, hw), w6 = b1[hw], w7 = prev1(b1, hw);
                        const uint32_t and8 = w0 & w1 & w2 & w3 & w4 & w5 & w6 & w7;
                        const uint32_t or8 = w0 | w1 | w2 | w3 | w4 | w5 | w6 | w7;
                        act = (or8 & ~and8) & em;
                        if (act) {
                            uint32_t sn = 0;
                            {
                                const int o0 = (hy - 1) * NW;
                                const uint32_t* xl = c.plane(hi, B_LOX);
                                const uint32_t* xh = c.plane(hi, B_HIX);
                                sn |= xl[o0 + hw] | prev1(xl + o0, hw) | xh[o0 + hw] | prev1(xh + o0, hw);
                                sn |= xl[o0 + NW + hw] | prev1(xl + o0 + NW, hw) | xh[o0 + NW + hw] |
                                      prev1(xh + o0 + NW, hw);
                            }
#pragma unroll
                            for (int pp = 0; pp < 2; ++pp) {
                                const int pls = pp ? hi : lo;
                                const uint32_t* yl = c.plane(pls, B_LOY) + hy * NW;
                                const uint32_t* yh = c.plane(pls, B_HIY) + hy * NW;
                                sn |= yl[hw] | prev1(yl, hw) | yh[hw] | prev1(yh, hw);
                                const uint32_t* zl0 = c.plane(pls, B_LOZ) + (hy - 1) * NW;
                                const uint32_t* zh0 = c.plane(pls, B_HIZ) + (hy - 1) * NW;
                                sn |= zl0[hw] | zl0[hw + NW] | zh0[hw] | zh0[hw + NW];
                            }
                            snp = act & sn;
                            fre = act & ~sn;
                            uint32_t bits = snp;
                            while (bits) {  // rare: cells with a vertex on a grid point
                                const int b = __ffs(bits) - 1;
                                bits &= bits - 1;
                                const int hc = 32 * hw + b;
                                const uint32_t cs = cell_case(c, L, hy, hc);
                                uint8_t ck[12];
                                cell_codes(c, L, hy, hc, c.estat[cs], true, ck);
                                const int8_t* tr = c.tri + cs * 15;
                                for (int k = 0; k < 15 && tr[k] >= 0; k += 3) {
                                    const uint8_t k0 = ck[tr[k]], k1 = ck[tr[k + 1]], k2 = ck[tr[k + 2]];
                                    if (k0 == k1 || k0 == k2 || k1 == k2) continue;
                                    const uint8_t kk[3] = {k0, k1, k2};
#pragma unroll
                                    for (int m = 0; m < 3; ++m) {
                                        const int corner = kk[m] >> 2, type = kk[m] & 3;
                                        const int rel = L + (corner >> 2);
                                        const int row = hy - 1 + ((corner >> 1) & 1);
                                        const int col = hc - 1 + (corner & 1);
                                        if (rel == 1 && row >= 1 && row <= c.Y1 - c.Y0 && col >= 32 &&
                                            col <= c.Z1 - c.Z0 + 31)
                                            atomicOr(&c.du[(type * c.RY + row) * NW + (col >> 5)],
                                                     1u << (col & 31));
                                    }
                                }
                            }
                        }
                    }
                    c.act[i] = act;
                    c.fre[i] = fre;
                    c.snp[i] = snp;
                    if (L == 0) c.fcnt[i] = 0;
                }
                __syncthreads();

                // T2: face counts of own cells (one lane per cell)
                iso::warp_foreach_bit(
                    warp * 32, RW, NWARP * 32, wscratch,
                    [&](int i) {
                        const int hy = (c.tbl[i] >> 16) & 0xff, hw = c.tbl[i] & 0xffff;
                        return (hy >= hyO0 && hy <= hyO1 && hw >= 1) ? (c.act[i] & c.ocell[hw]) : 0u;
                    },
                    [&](int i, int b) {
                        const int hy = (c.tbl[i] >> 16) & 0xff, hw = c.tbl[i] & 0xffff;
                        const uint32_t nt = cell_nfaces(c, 0, hy, 32 * hw + b, (c.snp[i] >> b) & 1u);
                        if (nt) atomicAdd(&c.fcnt[i], nt);
                    });
                // T3: vertex existence for the owned points (plane P)
                for (int i = tid; i < RW; i += BLOCK) {
                    const uint32_t x = c.tbl[i];
                    const int ly = (x >> 16) & 0xff, w = x & 0xffff;
                    uint32_t e0 = 0, e1 = 0, e2 = 0, e3 = 0;
                    const uint32_t om = (ly >= 1 && ly <= c.Y1 - c.Y0) ? c.ocol[w] : 0u;
                    if (om) {
                        const uint32_t* f0a = c.fre + ly * NW;
                        const uint32_t* f0b = f0a + NW;
                        const uint32_t* f1a = c.fre + RW + ly * NW;
                        const uint32_t* f1b = f1a + NW;
                        const uint32_t g0 = f0a[w], g0n = next1(f0a, w, NW), g1 = f0b[w],
                                       g1n = next1(f0b, w, NW);
                        const uint32_t h0 = f1a[w], h0n = next1(f1a, w, NW), h1 = f1b[w];
                        const int sB = c.sB;
                        const uint32_t* sgP = c.plane(sB, B_SGN) + ly * NW;
                        const bool rowok = c.rowoff[ly] >= 0;
                        // crossings of the edges keyed by plane P's points
                        const uint32_t zv = c.zval[w];
                        const uint32_t crx = (L0 && rowok) ? (sgP[w] ^ c.plane(c.sA, B_SGN)[i]) & zv : 0u;
                        const uint32_t cry = (rowok && ly >= 1 && c.rowoff[ly - 1] >= 0)
                                                 ? (sgP[w] ^ sgP[w - NW]) & zv : 0u;
                        const uint32_t crz = rowok ? (sgP[w] ^ prev1(sgP, w)) & zv & prev1(c.zval, w) : 0u;
                        uint32_t sn = c.plane(sB, B_LOX)[i] | c.plane(sB, B_HIX)[i];
                        e0 = crx & ~sn & ((g0 | g0n | g1 | g1n) | c.du[i]) & om;
                        sn = c.plane(sB, B_LOY)[i] | c.plane(sB, B_HIY)[i];
                        e1 = cry & ~sn & ((g0 | g0n | h0 | h0n) | c.du[RW + i]) & om;
                        sn = c.plane(sB, B_LOZ)[i] | c.plane(sB, B_HIZ)[i];
                        e2 = crz & ~sn & ((g0 | g1 | h0 | h1) | c.du[2 * RW + i]) & om;
                        e3 = c.du[3 * RW + i] & om;
                    }
                    c.ex[i] = e0;
                    c.ex[RW + i] = e1;
                    c.ex[2 * RW + i] = e2;
                    c.ex[3 * RW + i] = e3;
                    c.vcnt[i] = __popc(e0) + __popc(e1) + __popc(e2) + __popc(e3);
                }
                __syncthreads();

                // T4: warp 0 scans vertex and face counts, allocates staging.
                const long long tile = ((long long)P * c.nRT + c.rt) * c.nZT + c.zt;
                if (warp == 0) {
                    const int per = (RW + 31) / 32;
                    const int s0 = min(RW, lane * per), s1 = min(RW, s0 + per);
                    uint32_t sa = 0, sb = 0;
                    for (int k = s0; k < s1; ++k) { sa += c.vcnt[k]; sb += c.fcnt[k]; }
                    uint32_t ia = sa, ib = sb;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const uint32_t xa = __shfl_up_sync(~0u, ia, d), xb = __shfl_up_sync(~0u, ib, d);
                        if (lane >= d) { ia += xa; ib += xb; }
                    }
                    uint32_t ea = ia - sa, eb = ib - sb;
                    for (int k = s0; k < s1; ++k) {
                        const uint32_t xa = c.vcnt[k], xb = c.fcnt[k];
                        c.vcnt[k] = ea; c.fcnt[k] = eb;
                        ea += xa; eb += xb;
                    }
                    const uint32_t VT = __shfl_sync(~0u, ia, 31), FT = __shfl_sync(~0u, ib, 31);
                    if (lane == 0) {
                        // Staging is handed out in per-CTA blocks, so the global
                        // counters see one atomic per block rather than per tile.
                        // A tile of at least half a block gets an exact allocation;
                        // smaller ones share blocks, abandoning a remainder smaller
                        // than the tile (so at most half of any block is wasted).
                        auto take = [&](uint32_t n, unsigned long long blkn, unsigned long long* ctr,
                                        unsigned long long& cur, unsigned long long& end) {
                            if (2ull * n >= blkn) return atomicAdd(ctr, (unsigned long long)n);
                            if (cur + n > end) {
                                cur = atomicAdd(ctr, blkn);
                                end = cur + blkn;
                            }
                            const unsigned long long o = cur;
                            cur += n;
                            return o;
                        };
                        unsigned long long vo = 0, fo = 0;
                        if (VT) vo = take(VT, p.blkV, &p.ctr[1], c.misc[5], c.misc[6]);
                        if (FT) fo = take(FT, p.blkF, &p.ctr[2], c.misc[7], c.misc[8]);
                        if (tile / 1024 < p.nBlk) {
                            atomicAdd(&p.blk[2 * (tile / 1024)], (unsigned long long)VT);
                            atomicAdd(&p.blk[2 * (tile / 1024) + 1], (unsigned long long)FT);
                        }
                        c.misc[1] = vo;
                        c.misc[2] = fo;
                        c.misc[3] = VT;
                        c.misc[4] = FT;
                        McTileRec rec;
                        rec.vOff = uint32_t(vo);
                        rec.vCnt = VT;
                        rec.fOff = uint32_t(fo);
                        rec.fCnt = FT;
                        p.rec[tile] = rec;
                    }
                }
                __syncthreads();
                const unsigned long long vOff = c.misc[1], fOff = c.misc[2];
                const uint32_t VT = uint32_t(c.misc[3]), FT = uint32_t(c.misc[4]);
                const bool vfit = vOff + VT <= (unsigned long long)p.capSV;
                const bool ffit = fOff + FT <= (unsigned long long)p.capSF;
                if (tid == 0 && (!vfit || !ffit)) atomicCAS(p.status, 0, int(ISO_ERR_OVERFLOW));

                // T5a: staged vertices (position + key), one lane per point, in key order
                if (VT && vfit) {
                    iso::warp_foreach_bit(
                        warp * 32, RW, NWARP * 32, wscratch,
                        [&](int i) { return c.ex[i] | c.ex[RW + i] | c.ex[2 * RW + i] | c.ex[3 * RW + i]; },
                        [&](int i, int b) {
                            const uint32_t x = c.tbl[i];
                            const int ly = (x >> 16) & 0xff, w = x & 0xffff;
                            const uint32_t e[4] = {c.ex[i], c.ex[RW + i], c.ex[2 * RW + i], c.ex[3 * RW + i]};
                            const uint32_t below = (1u << b) - 1u;
                            unsigned long long o = vOff + c.vcnt[i] + __popc(e[0] & below) +
                                                   __popc(e[1] & below) + __popc(e[2] & below) +
                                                   __popc(e[3] & below);
                            const int col = 32 * w + b;
                            const int sB = c.sB;
                            const float bx = c.gx[sB], by = c.gy[ly], bz = c.gz[col];
                            const bool edge = ((e[0] | e[1] | e[2]) >> b) & 1u;
                            const float vb = edge ? c.value(P, ly, col) : 0.0f;
#pragma unroll
                            for (int type = 0; type < 4; ++type) {
                                if (!((e[type] >> b) & 1u)) continue;
                                float px = bx, py = by, pz = bz;
                                if (type < 3) {
                                    const int pa = type == 0 ? P - 1 : P;
                                    const int ra = type == 1 ? ly - 1 : ly;
                                    const int ca = type == 2 ? col - 1 : col;
                                    const float va = c.value(pa, ra, ca);
                                    const float t = iso::cross_t(c.level, va, vb);
                                    px = iso::lerp1(t, type == 0 ? c.gx[c.sA] : bx, bx);
                                    py = iso::lerp1(t, c.gy[ra], by);
                                    pz = iso::lerp1(t, c.gz[ca], bz);
                                }
                                const uint32_t key = (uint32_t((ly - 1) * c.ZC + (col - 32)) << 2) | type;
                                p.sv[o++] = make_float4(px, py, pz, __uint_as_float(key));
                            }
                        });
                }
                // T5b: staged faces of own cells, one lane per cell, in cell order
                if (FT && ffit) {
                    iso::warp_foreach_bit(
                        warp * 32, RW, NWARP * 32, wscratch,
                        [&](int i) {
                            const int hy = (c.tbl[i] >> 16) & 0xff, hw = c.tbl[i] & 0xffff;
                            return (hy >= hyO0 && hy <= hyO1 && hw >= 1) ? (c.act[i] & c.ocell[hw]) : 0u;
                        },
                        [&](int i, int b) {
                            const int hy = (c.tbl[i] >> 16) & 0xff, hw = c.tbl[i] & 0xffff;
                            const uint32_t own = c.act[i] & c.ocell[hw];
                            const uint32_t snp = c.snp[i];
                            // faces of the word's earlier own cells come first
                            unsigned long long o = fOff + c.fcnt[i];
                            uint32_t prior = own & ((1u << b) - 1u);
                            while (prior) {
                                const int b2 = __ffs(prior) - 1;
                                prior &= prior - 1;
                                o += cell_nfaces(c, 0, hy, 32 * hw + b2, (snp >> b2) & 1u);
                            }
                            const int hc = 32 * hw + b;
                            const uint32_t cs = cell_case(c, 0, hy, hc);
                            const bool sn = (snp >> b) & 1u;
                            uint8_t ck[12];
                            cell_codes(c, 0, hy, hc, c.estat[cs], sn, ck);
                            // owner-relative references of the 8 corner points
                            uint32_t base[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                const int rel = k >> 2;
                                const int row = hy - 1 + ((k >> 1) & 1);
                                const int col = hc - 1 + (k & 1);
                                const int drt = row == 0, dzt = col == 31;
                                const uint32_t lrow = uint32_t(row - 1 + drt * c.R);
                                const uint32_t lcol = uint32_t(col - 32 + dzt * c.ZC);
                                const uint32_t slot = uint32_t((1 - rel) * 4 + drt * 2 + dzt);
                                base[k] = (slot << 24) | ((lrow * uint32_t(c.ZC) + lcol) << 2);
                            }
                            const int8_t* tr = c.tri + cs * 15;
                            for (int k = 0; k < 15 && tr[k] >= 0; k += 3) {
                                const uint8_t k0 = ck[tr[k]], k1 = ck[tr[k + 1]], k2 = ck[tr[k + 2]];
                                if (sn && (k0 == k1 || k0 == k2 || k1 == k2)) continue;
                                uint32_t* dst = p.sf + 3 * o++;
                                dst[0] = base[k0 >> 2] | (k0 & 3u);
                                dst[1] = base[k1 >> 2] | (k1 & 3u);
                                dst[2] = base[k2 >> 2] | (k2 & 3u);
                            }
                        });
                }
                for (int i = tid; i < RW; i += BLOCK) {
                    c.du[i] = 0;
                    c.du[RW + i] = 0;
                    c.du[2 * RW + i] = 0;
                    c.du[3 * RW + i] = 0;
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

// Sign bitmap of the whole grid: bit z % 32 of word [(x * ny + y) * NWg + z / 32]
// is (v - level < 0).  One warp per grid row, all of the row's loads in flight
// before the ballots; lane w keeps word w so each 32 words leave in one store.
constexpr int SIGN_BLOCK = 256;
constexpr int SIGN_UNROLL = 16;

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

// Exclusive prefix of per-tile counts: CTA b scans tiles [1024 b, 1024 b + 1024)
// and adds the totals of earlier blocks (accumulated by the extract kernel).
__global__ void __launch_bounds__(1024) mc_tile_scan(const McTileRec* __restrict__ rec, uint2* pre,
                                                     const unsigned long long* __restrict__ blk,
                                                     long long n, long long nBlk, long long* counts,
                                                     int* status, long long capV, long long capF) {
    __shared__ unsigned long long wa[32], wb[32];
    __shared__ unsigned long long base[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long b = blockIdx.x;
    // prefix of earlier blocks
    unsigned long long pa = 0, pb = 0;
    for (long long k = tid; k < b; k += 1024) { pa += blk[2 * k]; pb += blk[2 * k + 1]; }
    for (int d = 16; d >= 1; d >>= 1) {
        pa += __shfl_down_sync(~0u, pa, d);
        pb += __shfl_down_sync(~0u, pb, d);
    }
    if (lane == 0) { wa[warp] = pa; wb[warp] = pb; }
    __syncthreads();
    if (warp == 0) {
        unsigned long long x = wa[lane], y = wb[lane];
        for (int d = 16; d >= 1; d >>= 1) {
            x += __shfl_down_sync(~0u, x, d);
            y += __shfl_down_sync(~0u, y, d);
        }
        if (lane == 0) { base[0] = x; base[1] = y; }
    }
    __syncthreads();
    const long long i = b * 1024 + tid;
    unsigned long long a = 0, c = 0;
    if (i < n) { const McTileRec r = rec[i]; a = r.vCnt; c = r.fCnt; }
    unsigned long long ia = a, ic = c;
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long xa = __shfl_up_sync(~0u, ia, d), xc = __shfl_up_sync(~0u, ic, d);
        if (lane >= d) { ia += xa; ic += xc; }
    }
    if (lane == 31) { wa[warp] = ia; wb[warp] = ic; }
    __syncthreads();
    if (warp == 0) {
        unsigned long long va = wa[lane], vc = wb[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long xa = __shfl_up_sync(~0u, va, d), xc = __shfl_up_sync(~0u, vc, d);
            if (lane >= d) { va += xa; vc += xc; }
        }
        wa[lane] = va;
        wb[lane] = vc;
    }
    __syncthreads();
    const unsigned long long ea = base[0] + (warp ? wa[warp - 1] : 0ull) + ia - a;
    const unsigned long long ec = base[1] + (warp ? wb[warp - 1] : 0ull) + ic - c;
    if (i < n) pre[i] = make_uint2(uint32_t(ea), uint32_t(ec));
    if (b == nBlk - 1 && tid == 1023) {
        const long long V = (long long)(base[0] + wa[31]), F = (long long)(base[1] + wb[31]);
        counts[0] = V;
        counts[1] = F;
        if (V > capV || F > capF) atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
    }
}

// Final vertices and faces; one warp per tile.  Face references are resolved by
// binary search in the key lists of the (up to 8) tiles they can point to.
constexpr int RES_BLOCK = 256;
constexpr int RES_KCAP = 512;  // staged keys per warp

__global__ void __launch_bounds__(RES_BLOCK) mc_resolve(const McParams p) {
    const McTiles& T = p.t;
    __shared__ uint32_t keys_all[RES_BLOCK / 32][RES_KCAP];
    __shared__ uint32_t seg_all[RES_BLOCK / 32][4][8];  // len, off, base, voff per slot
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* keys = keys_all[warp];
    uint32_t(*seg)[8] = seg_all[warp];
    const long long stride = (long long)gridDim.x * (RES_BLOCK / 32);
    for (long long tile = (long long)blockIdx.x * (RES_BLOCK / 32) + warp; tile < T.nTiles;
         tile += stride) {
        const McTileRec rec = p.rec[tile];
        if (rec.vCnt == 0 && rec.fCnt == 0) continue;
        const uint2 pre = p.pre[tile];
        const bool vfit = (unsigned long long)rec.vOff + rec.vCnt <= (unsigned long long)p.capSV;
        const bool ffit = (unsigned long long)rec.fOff + rec.fCnt <= (unsigned long long)p.capSF;
        for (uint32_t i = lane; i < rec.vCnt && vfit; i += 32) {
            const long long o = (long long)pre.x + i;
            if (o >= p.capV) break;
            const float4 v = p.sv[rec.vOff + i];
            p.vout[3 * o + 0] = v.x;
            p.vout[3 * o + 1] = v.y;
            p.vout[3 * o + 2] = v.z;
        }
        if (rec.fCnt == 0 || !ffit) continue;
        // neighbour key lists: lane sl < 8 reads slot sl (plane, row group,
        // z chunk one step back per bit)
        const int zt = int(tile % T.nZT);
        const int rt = int((tile / T.nZT) % T.nRT);
        const int P = int(tile / ((long long)T.nZT * T.nRT));
        uint32_t sLen = 0, sBase = 0, sVOff = 0;
        if (lane < 8) {
            const int pp = P - (lane >> 2), rr = rt - ((lane >> 1) & 1), zz = zt - (lane & 1);
            if (pp >= 0 && rr >= 0 && zz >= 0) {
                const long long t2 = ((long long)pp * T.nRT + rr) * T.nZT + zz;
                const McTileRec r2 = p.rec[t2];
                if ((unsigned long long)r2.vOff + r2.vCnt <= (unsigned long long)p.capSV) {
                    sLen = r2.vCnt;
                    sVOff = r2.vOff;
                    sBase = p.pre[t2].x;
                }
            }
        }
        uint32_t incl = sLen;
        for (int d = 1; d < 8; d <<= 1) {
            const uint32_t x = __shfl_up_sync(~0u, incl, d);
            if (lane >= d) incl += x;
        }
        const uint32_t total = __shfl_sync(~0u, incl, 7);
        const uint32_t sOff = incl - sLen;
        const bool staged = total <= RES_KCAP;
        if (lane < 8) {
            seg[0][lane] = sLen;
            seg[1][lane] = sOff;
            seg[2][lane] = sBase;
            seg[3][lane] = sVOff;
        }
        if (staged) {
            for (int sl = 0; sl < 8; ++sl) {
                const uint32_t len = __shfl_sync(~0u, sLen, sl), off = __shfl_sync(~0u, sOff, sl);
                const uint32_t vo = __shfl_sync(~0u, sVOff, sl);
                for (uint32_t i = lane; i < len; i += 32) keys[off + i] = __float_as_uint(p.sv[vo + i].w);
            }
        }
        __syncwarp();
        for (uint32_t f = lane; f < rec.fCnt; f += 32) {
            const long long o = (long long)pre.y + f;
            if (o >= p.capF) break;
            const uint32_t* src = p.sf + 3ull * (rec.fOff + f);
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const uint32_t ref = src[m];
                const int sl = int(ref >> 24);
                const uint32_t local = ref & 0xffffffu;
                const uint32_t segLen = seg[0][sl], segOff = seg[1][sl];
                const uint32_t segBase = seg[2][sl], segVOff = seg[3][sl];
                uint32_t lo = 0, hi = segLen;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    const uint32_t k = staged ? keys[segOff + mid] : __float_as_uint(p.sv[segVOff + mid].w);
                    if (k < local) lo = mid + 1; else hi = mid;
                }
                const uint32_t k = lo < segLen ? (staged ? keys[segOff + lo]
                                                         : __float_as_uint(p.sv[segVOff + lo].w))
                                               : 0xffffffffu;
                int idx;
                if (k == local) {
                    idx = int(segBase + lo);
                } else {
                    atomicCAS(p.status, 0, int(ISO_ERR_LOOKUP));
                    idx = -1;
                }
                p.fout[3 * o + m] = idx;
            }
        }
        __syncwarp();
    }
}

template <int BLOCK>
int launch_extract(const McParams& p, cudaStream_t st) {
    auto k = mc_extract<BLOCK>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p.t.smemBytes));
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, BLOCK, p.t.smemBytes) != cudaSuccess ||
        per < 1)
        per = 1;
    per = std::min(per, std::max(1, p.t.ctasPerSm));  // staging slack assumes at most this many
    long long grid = (long long)sms * per;
    if (grid > p.t.nItems) grid = p.t.nItems;
    if (grid < 1) grid = 1;
    k<<<unsigned(grid), BLOCK, p.t.smemBytes, st>>>(p);
    return cudaGetLastError() == cudaSuccess ? 0 : ISO_ERR_CUDA;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host API

void mc_signs_launch(const float* vals, int nx, int ny, int nz, float level, uint32_t* out,
                     cudaStream_t st) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long rows = (long long)nx * ny;
    const long long want = (rows + (SIGN_BLOCK / 32) - 1) / (SIGN_BLOCK / 32);
    const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sms * 32));
    mc_signs<<<unsigned(grid), SIGN_BLOCK, 0, st>>>(vals, rows, nz, level, out);
}

int mc_plan_tiles(int nx, int ny, int nz, int rows, int slabs, int threads, int zchunk,
                  int sm_count, McTiles* out) {
    McTiles t{};
    t.nx = nx; t.ny = ny; t.nz = nz;
    t.S = std::max(4, slabs);
    t.threads = threads == 512 ? 512 : 256;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        optin <= 0)
        optin = 227 * 1024;
    // small footprints keep several CTAs resident per SM
    const size_t budget = std::min(size_t(optin) - 2048, size_t(96) * 1024);
    // Full-z tiles when they fit with at least one row; else z chunks of one row.
    int R = std::max(1, rows);
    int ZC = (nz + 31) / 32 * 32;
    if (zchunk > 0 && zchunk < ZC) ZC = std::max(32, zchunk / 32 * 32);
    auto fits = [&](int r, int zc) {
        McTiles u = t;
        u.R = r; u.ZC = zc; u.RY = r + 2; u.NW = zc / 32 + 2; u.CZP = 0;
        // rows and words must fit the 8/16-bit fields of the decode table
        return r + 2 <= 255 && u.NW <= 0xffff && make_layout(u).total <= budget;
    };
    while (R > 1 && !fits(R, ZC)) --R;
    if (!fits(R, ZC)) {
        R = 1;
        while (ZC > 32 && !fits(1, ZC)) ZC -= 32;
        if (!fits(1, ZC)) return ISO_ERR_ARG;
    }
    if (ZC < nz) R = 1;  // split z => one row per tile keeps tiles contiguous
    t.R = R; t.ZC = ZC;
    t.RY = R + 2; t.NW = ZC / 32 + 2; t.CZP = 0;
    t.nRT = (ny + R - 1) / R;
    t.nZT = (nz + ZC - 1) / ZC;
    t.nTiles = (long long)nx * t.nRT * t.nZT;
    if ((long long)R * ZC * 4 >= (1ll << 24)) return ISO_ERR_ARG;
    const Layout L = make_layout(t);
    t.smemBytes = L.total;
    {
        int per = 0;
        cudaError_t e;
        if (t.threads == 512) {
            cudaFuncSetAttribute(mc_extract<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.total));
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mc_extract<512>, 512, L.total);
        } else {
            cudaFuncSetAttribute(mc_extract<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.total));
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, mc_extract<256>, 256, L.total);
        }
        t.ctasPerSm = (e == cudaSuccess && per > 0) ? per : 1;
    }
    // Work items: aim for several per CTA.
    long long cols = (long long)t.nRT * t.nZT;
    long long ctas = (long long)std::max(1, sm_count) * t.ctasPerSm;
    long long want = 4 * ctas;
    int chunks = int(std::min<long long>(nx, std::max<long long>(1, (want + cols - 1) / cols)));
    t.PC = (nx + chunks - 1) / chunks;
    t.nChunks = (nx + t.PC - 1) / t.PC;
    t.nItems = (long long)t.nChunks * cols;
    *out = t;
    return 0;
}

// Bound on t for an edge vertex to round onto an endpoint.  For the varying
// coordinate, (1 - t) * a + t * b rounds to a only if t * |b - a| is within a few
// ulps of max(|a|, |b|): t <= ~5 * 2^-24 * (|a| + |b|) / h, h the grid spacing.
// tau = 2^-20 * (1 + max |coord| / h) keeps a 1.6x margin on that bound; the
// same holds for 1 - t.
float mc_snap_tau(const float amin[3], const float amax[3], const int n[3]) {
    double r = 0;
    for (int k = 0; k < 3; ++k) {
        double size = double(amax[k]) - double(amin[k]);
        double m = std::max(std::fabs(double(amin[k])), std::fabs(double(amax[k])));
        if (size == 0.0 || !std::isfinite(size)) return 1.0f;
        r = std::max(r, m * double(std::max(n[k] - 1, 1)) / std::fabs(size));
    }
    double tau = std::ldexp(1.0, -20) * (1.0 + r);
    return tau >= 0.5 ? 1.0f : float(tau);
}

// Staging blocks handed to a CTA at a time, and the slack they can leave unused.
static void staging_blocks(const McTiles& t, long long capV, long long capF, unsigned long long* bv,
                           unsigned long long* bf, long long* slackV, long long* slackF) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ctas = (long long)sms * std::max(1, t.ctasPerSm);  // resident extract CTAs
    *bv = (unsigned long long)std::min<long long>(4096, std::max<long long>(64, capV / (4 * ctas) + 1));
    *bf = (unsigned long long)std::min<long long>(8192, std::max<long long>(64, capF / (4 * ctas) + 1));
    // block waste is below half of the block-allocated total, plus one open
    // block per CTA: capacity 2 * cap + ctas * block is always enough
    *slackV = capV + ctas * (long long)*bv;
    *slackF = capF + ctas * (long long)*bf;
    (void)t;
}

size_t mc_workspace_bytes(const McTiles& t, long long capV, long long capF) {
    unsigned long long bv, bf;
    long long sv, sf;
    staging_blocks(t, capV, capF, &bv, &bf, &sv, &sf);
    const long long nBlk = (t.nTiles + 1023) / 1024;
    size_t o = 0;
    o = al16(o + size_t(t.nTiles) * sizeof(McTileRec));
    o = al16(o + size_t(t.nTiles) * sizeof(uint2));
    o = al16(o + size_t(std::max<long long>(capV + sv, 1)) * sizeof(float4));
    o = al16(o + size_t(std::max<long long>(capF + sf, 1)) * 3 * sizeof(uint32_t));
    o = al16(o + size_t(nBlk) * 2 * sizeof(unsigned long long));
    o = al16(o + 4 * sizeof(unsigned long long));
    o = al16(o + size_t(t.nx) * t.ny * ((t.nz + 31) / 32) * sizeof(uint32_t));
    return o + 256;
}

int mc_launch(const McParams& p0, void* ws, size_t ws_bytes, cudaStream_t st) {
    McParams p = p0;
    const McTiles& t = p.t;
    const size_t need = mc_workspace_bytes(t, p.capV, p.capF);
    if (ws_bytes < need) return ISO_ERR_WORKSPACE;
    long long slackV, slackF;
    staging_blocks(t, p.capV, p.capF, &p.blkV, &p.blkF, &slackV, &slackF);
    p.nBlk = (t.nTiles + 1023) / 1024;
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    p.rec = reinterpret_cast<McTileRec*>(b + o); o = al16(o + size_t(t.nTiles) * sizeof(McTileRec));
    p.pre = reinterpret_cast<uint2*>(b + o);     o = al16(o + size_t(t.nTiles) * sizeof(uint2));
    p.capSV = p.capV + slackV;
    p.capSF = p.capF + slackF;
    p.sv = reinterpret_cast<float4*>(b + o);     o = al16(o + size_t(std::max<long long>(p.capSV, 1)) * sizeof(float4));
    p.sf = reinterpret_cast<uint32_t*>(b + o);   o = al16(o + size_t(std::max<long long>(p.capSF, 1)) * 3 * sizeof(uint32_t));
    p.blk = reinterpret_cast<unsigned long long*>(b + o); o = al16(o + size_t(p.nBlk) * 2 * sizeof(unsigned long long));
    p.ctr = reinterpret_cast<unsigned long long*>(b + o); o = al16(o + 4 * sizeof(unsigned long long));
    p.signs = reinterpret_cast<uint32_t*>(b + o);
    if (cudaMemsetAsync(p.blk, 0, size_t(p.nBlk) * 2 * sizeof(unsigned long long) + 64, st) !=
        cudaSuccess)
        return ISO_ERR_CUDA;
    if (cudaMemsetAsync(p.ctr, 0, 4 * sizeof(unsigned long long), st) != cudaSuccess)
        return ISO_ERR_CUDA;
    if (t.nTiles > 0x7fffffffll) return ISO_ERR_ARG;
    {
        iso::ProfScope ps("mc_signs", st);
        mc_signs_launch(p.vals, t.nx, t.ny, t.nz, p.level, p.signs, st);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    {
        iso::ProfScope ps("mc_extract", st);
        int rc = t.threads == 512 ? launch_extract<512>(p, st) : launch_extract<256>(p, st);
        if (rc) return rc;
    }
    {
        iso::ProfScope ps("mc_tile_scan", st);
        mc_tile_scan<<<unsigned(p.nBlk), 1024, 0, st>>>(p.rec, p.pre, p.blk, t.nTiles, p.nBlk, p.counts,
                                                       p.status, p.capV, p.capF);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    {
        iso::ProfScope ps("mc_resolve", st);
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long want = (t.nTiles + (RES_BLOCK / 32) - 1) / (RES_BLOCK / 32);
        const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sms * 8));
        mc_resolve<<<unsigned(grid), RES_BLOCK, 0, st>>>(p);
        if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    }
    return 0;
}
