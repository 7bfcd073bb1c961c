// Dense-grid marching cubes on sm_103a.
//
// Three launches on one stream:
//   1. mc_extract  persistent CTAs; each work item is a column of tiles
//                  (row group, z chunk) swept along x over a chunk of planes.
//                  Point slabs (one plane x (R+2) rows x (ZC+2) z) stream into a
//                  shared-memory ring by TMA bulk copies, so every grid value
//                  is read from HBM once.  Per slab: sign bits (warp ballot),
//                  crossed-edge bitmaps and "snap" bitmaps (edge vertices that
//                  round exactly onto a grid point).  Per tile: cell activity
//                  by word-wide bit logic, face counts, vertex existence, and
//                  staged vertices (position + key) and faces (key references).
//   2. mc_tile_scan  exclusive prefix of per-tile vertex / face counts.
//   3. mc_resolve  copies staged vertices to their final slots and turns face
//                  key references into vertex indices.
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
#include <cstdio>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "mc_dense.cuh"

namespace {

constexpr int NB = 10;  // bitmaps kept per slab
enum { B_SGN = 0, B_CRX, B_CRY, B_CRZ, B_LOX, B_LOY, B_LOZ, B_HIX, B_HIY, B_HIZ };

struct Layout {
    size_t vals, bm, act, fre, snp, du, ex, vcnt, fcnt, gx, gy, gz, sh, zval, ecol, ocol, ocell,
        estat, tri, ntri, bar, misc, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline Layout make_layout(const McTiles& t) {
    Layout L;
    size_t o = 0;
    const size_t rw = size_t(t.RY) * t.NW;  // words per bitmap
    L.vals = o;  o = al16(o + size_t(t.S) * t.RY * t.CZP * 4);
    L.bm = o;    o = al16(o + size_t(t.S) * NB * rw * 4);
    L.act = o;   o = al16(o + 2 * rw * 4);
    L.fre = o;   o = al16(o + 2 * rw * 4);
    L.snp = o;   o = al16(o + 2 * rw * 4);
    L.du = o;    o = al16(o + 4 * rw * 4);
    L.ex = o;    o = al16(o + 4 * rw * 4);
    L.vcnt = o;  o = al16(o + rw * 4);
    L.fcnt = o;  o = al16(o + rw * 4);
    L.gx = o;    o = al16(o + size_t(t.S) * 4);
    L.gy = o;    o = al16(o + size_t(t.RY) * 4);
    L.gz = o;    o = al16(o + size_t(32) * t.NW * 4);
    L.sh = o;    o = al16(o + size_t(t.S) * t.RY * 4);
    L.zval = o;  o = al16(o + size_t(t.NW) * 4);
    L.ecol = o;  o = al16(o + size_t(t.NW) * 4);
    L.ocol = o;  o = al16(o + size_t(t.NW) * 4);
    L.ocell = o; o = al16(o + size_t(t.NW) * 4);
    L.estat = o; o = al16(o + 256 * 2);
    L.tri = o;   o = al16(o + 256 * 15);
    L.ntri = o;  o = al16(o + 256);
    L.bar = o;   o = al16(o + size_t(t.S) * 8);
    L.misc = o;  o = al16(o + 64);
    L.total = o;
    return L;
}

// Per-CTA view of shared memory.
struct Sh {
    float* vals;
    uint32_t* bm;
    uint32_t *act, *fre, *snp, *du, *ex, *vcnt, *fcnt;
    float *gx, *gy, *gz;
    int* sh;
    uint32_t *zval, *ecol, *ocol, *ocell;
    uint16_t* estat;
    int8_t* tri;
    uint8_t* ntri;
    uint64_t* bar;
    unsigned long long* misc;
};

// Block-wide exclusive scan of two uint32 arrays of length n in place.
// Returns the totals through out[0], out[1] (valid for all threads after the call).
template <int BLOCK>
__device__ void scan2(uint32_t* a, uint32_t* b, int n, uint32_t* tmp /*2*BLOCK/32+2*/,
                      uint32_t& ta, uint32_t& tb) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARP = BLOCK / 32;
    const int per = (n + BLOCK - 1) / BLOCK;
    const int s0 = min(n, tid * per), s1 = min(n, s0 + per);
    uint32_t sa = 0, sb = 0;
    for (int i = s0; i < s1; ++i) { sa += a[i]; sb += b[i]; }
    uint32_t ia = sa, ib = sb;
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t xa = __shfl_up_sync(~0u, ia, d), xb = __shfl_up_sync(~0u, ib, d);
        if (lane >= d) { ia += xa; ib += xb; }
    }
    if (lane == 31) { tmp[warp] = ia; tmp[NWARP + warp] = ib; }
    __syncthreads();
    if (warp == 0) {
        uint32_t va = lane < NWARP ? tmp[lane] : 0u, vb = lane < NWARP ? tmp[NWARP + lane] : 0u;
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t xa = __shfl_up_sync(~0u, va, d), xb = __shfl_up_sync(~0u, vb, d);
            if (lane >= d) { va += xa; vb += xb; }
        }
        if (lane < NWARP) { tmp[lane] = va; tmp[NWARP + lane] = vb; }
        if (lane == NWARP - 1) { tmp[2 * NWARP] = va; tmp[2 * NWARP + 1] = vb; }
    }
    __syncthreads();
    uint32_t ea = (warp ? tmp[warp - 1] : 0u) + ia - sa;
    uint32_t eb = (warp ? tmp[NWARP + warp - 1] : 0u) + ib - sb;
    for (int i = s0; i < s1; ++i) {
        uint32_t xa = a[i], xb = b[i];
        a[i] = ea; b[i] = eb;
        ea += xa; eb += xb;
    }
    ta = tmp[2 * NWARP];
    tb = tmp[2 * NWARP + 1];
    __syncthreads();
}

using iso::bit_at;
using iso::next1;
using iso::prev1;

struct Ctx {
    // grid
    int nx, ny, nz;
    float level;
    // tiling
    int R, ZC, RY, NW, CZP, nRT, nZT;
    // current item / tile
    int rt, zt, Y0, Y1, Z0, Z1;
    int P, sA, sB, sC;  // slab slots of planes P-1, P, P+1 (-1 when absent)
};

__device__ __forceinline__ const uint32_t* bmrow(const Sh& s, const Ctx& c, int slot, int arr,
                                                 int row) {
    return s.bm + ((size_t(slot) * NB + arr) * c.RY + row) * c.NW;
}
__device__ __forceinline__ float valat(const Sh& s, const Ctx& c, int slot, int row, int col) {
    int r = slot * c.RY + row;
    return s.vals[size_t(r) * c.CZP + col - 28 + s.sh[r]];
}

// Case number of the cell whose highest corner is (row hy, column hc) in
// layer L (0: planes P-1..P, 1: planes P..P+1).
__device__ __forceinline__ uint32_t cell_case(const Sh& s, const Ctx& c, int L, int hy, int hc) {
    int lo = L ? c.sB : c.sA, hi = L ? c.sC : c.sB;
    uint32_t cs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int pl = (k >> 2) ? hi : lo;
        int row = hy - 1 + ((k >> 1) & 1);
        int col = hc - 1 + (k & 1);
        cs |= bit_at(bmrow(s, c, pl, B_SGN, row), col) << k;
    }
    return cs;
}

// Keys of the crossed edges of a cell (L, hy, hc).  Key layout:
// ((rel * RY + row) * (32 * NW) + col) * 4 + type, rel = plane - (P - 1),
// type 0/1/2 = edge along x/y/z keyed by its high endpoint, 3 = grid point.
__device__ __forceinline__ void cell_keys(const Sh& s, const Ctx& c, int L, int hy, int hc,
                                          uint32_t est, uint32_t* key) {
    const int CW = 32 * c.NW;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        if (!((est >> e) & 1u)) continue;
        int a = ISO_EDGE_CORNERS[2 * e], b = ISO_EDGE_CORNERS[2 * e + 1];
        int d = b - a;
        int ax = d == 4 ? 0 : (d == 2 ? 1 : 2);
        int relb = L + (b >> 2), rowb = hy - 1 + ((b >> 1) & 1), colb = hc - 1 + (b & 1);
        int slot = relb == 0 ? c.sA : (relb == 1 ? c.sB : c.sC);
        uint32_t lo = bit_at(bmrow(s, c, slot, B_LOX + ax, rowb), colb);
        uint32_t hi = bit_at(bmrow(s, c, slot, B_HIX + ax, rowb), colb);
        int rel = relb, row = rowb, col = colb, type = ax;
        if (lo) {
            rel = L + (a >> 2); row = hy - 1 + ((a >> 1) & 1); col = hc - 1 + (a & 1); type = 3;
        } else if (hi) {
            type = 3;
        }
        key[e] = ((uint32_t(rel) * c.RY + row) * CW + col) * 4u + type;
    }
}

__device__ __forceinline__ void key_split(const Ctx& c, uint32_t k, int& rel, int& row, int& col,
                                          int& type) {
    const int CW = 32 * c.NW;
    type = k & 3u;
    k >>= 2;
    col = k % CW;
    k /= CW;
    row = k % c.RY;
    rel = k / c.RY;
}

__device__ __forceinline__ bool key_owned(const Ctx& c, int rel, int row, int col) {
    return rel == 1 && row >= 1 && row <= c.Y1 - c.Y0 && col >= 32 && col <= c.Z1 - c.Z0 + 31;
}

// Face reference to the tile owning a key: (slot << 24) | local key.
__device__ __forceinline__ uint32_t key_ref(const Ctx& c, uint32_t k) {
    int rel, row, col, type;
    key_split(c, k, rel, row, col, type);
    int py = c.Y0 - 1 + row, pz = c.Z0 - 32 + col;
    int drt = py < c.Y0 ? 1 : 0, dzt = pz < c.Z0 ? 1 : 0;
    int y0 = c.Y0 - drt * c.R, z0 = c.Z0 - dzt * c.ZC;
    uint32_t local = (uint32_t((py - y0) * c.ZC + (pz - z0)) << 2) | uint32_t(type);
    uint32_t slot = uint32_t((1 - rel) * 4 + drt * 2 + dzt);
    return (slot << 24) | local;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) mc_extract(const McParams p) {
    extern __shared__ __align__(128) uint8_t smem[];
    const McTiles& T = p.t;
    const Layout LY = make_layout(T);
    Sh s;
    s.vals = reinterpret_cast<float*>(smem + LY.vals);
    s.bm = reinterpret_cast<uint32_t*>(smem + LY.bm);
    s.act = reinterpret_cast<uint32_t*>(smem + LY.act);
    s.fre = reinterpret_cast<uint32_t*>(smem + LY.fre);
    s.snp = reinterpret_cast<uint32_t*>(smem + LY.snp);
    s.du = reinterpret_cast<uint32_t*>(smem + LY.du);
    s.ex = reinterpret_cast<uint32_t*>(smem + LY.ex);
    s.vcnt = reinterpret_cast<uint32_t*>(smem + LY.vcnt);
    s.fcnt = reinterpret_cast<uint32_t*>(smem + LY.fcnt);
    s.gx = reinterpret_cast<float*>(smem + LY.gx);
    s.gy = reinterpret_cast<float*>(smem + LY.gy);
    s.gz = reinterpret_cast<float*>(smem + LY.gz);
    s.sh = reinterpret_cast<int*>(smem + LY.sh);
    s.zval = reinterpret_cast<uint32_t*>(smem + LY.zval);
    s.ecol = reinterpret_cast<uint32_t*>(smem + LY.ecol);
    s.ocol = reinterpret_cast<uint32_t*>(smem + LY.ocol);
    s.ocell = reinterpret_cast<uint32_t*>(smem + LY.ocell);
    s.estat = reinterpret_cast<uint16_t*>(smem + LY.estat);
    s.tri = reinterpret_cast<int8_t*>(smem + LY.tri);
    s.ntri = reinterpret_cast<uint8_t*>(smem + LY.ntri);
    s.bar = reinterpret_cast<uint64_t*>(smem + LY.bar);
    s.misc = reinterpret_cast<unsigned long long*>(smem + LY.misc);
    __shared__ uint32_t scan_tmp[2 * (BLOCK / 32) + 2];
    __shared__ int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARP = BLOCK / 32;

    Ctx c;
    c.nx = T.nx; c.ny = T.ny; c.nz = T.nz; c.level = p.level;
    c.R = T.R; c.ZC = T.ZC; c.RY = T.RY; c.NW = T.NW; c.CZP = T.CZP;
    c.nRT = T.nRT; c.nZT = T.nZT;
    const int S = T.S;
    const int RW = c.RY * c.NW;

    // Lookup tables.
    for (int i = tid; i < 256; i += BLOCK) {
        s.estat[i] = ISO_EDGE_STATUS[i];
        int n = 0;
        if (p.method == 0) {
            while (n < ISO_NAGAE_MAX_TRI && ISO_TRI_NAGAE[i * 15 + 3 * n] >= 0) ++n;
        } else {
            while (n < ISO_LORENSEN_MAX_TRI && ISO_TRI_LORENSEN[i * 12 + 3 * n] >= 0) ++n;
        }
        s.ntri[i] = uint8_t(n);
    }
    for (int i = tid; i < 256 * 15; i += BLOCK) {
        int cs = i / 15, k = i % 15;
        s.tri[i] = p.method == 0 ? ISO_TRI_NAGAE[i] : (k < 12 ? ISO_TRI_LORENSEN[cs * 12 + k] : -1);
    }
    if (tid == 0) {
        for (int k = 0; k < S; ++k) iso::mbar_init(&s.bar[k], 1);
        iso::mbar_init_fence();
        s_abort = 0;
    }
    __syncthreads();

    unsigned long long qbase = 0;  // slabs loaded by this CTA before the current item
    const long long perChunk = (long long)c.nRT * c.nZT;

    for (;;) {
        if (tid == 0) s.misc[0] = atomicAdd(&p.ctr[0], 1ull);
        __syncthreads();
        const long long item = (long long)s.misc[0];
        if (item >= T.nItems) break;
        const int chunk = int(item / perChunk);
        const int col = int(item % perChunk);
        c.rt = col / c.nZT;
        c.zt = col % c.nZT;
        c.Y0 = c.rt * c.R;
        c.Y1 = min(c.Y0 + c.R, c.ny);
        c.Z0 = c.zt * c.ZC;
        c.Z1 = min(c.Z0 + c.ZC, c.nz);
        const int Pa = chunk * T.PC, Pb = min(Pa + T.PC, c.nx);
        const int pfirst = max(Pa - 1, 0), plast = min(Pb, c.nx - 1);
        const int nslab = plast - pfirst + 1;

        // Per-item tables: coordinates and column masks.
        const int zf = max(c.Z0 - 1, 0), zl = min(c.Z1, c.nz - 1);  // loaded z range
        for (int i = tid; i < 32 * c.NW; i += BLOCK) {
            int z = c.Z0 - 32 + i;
            s.gz[i] = (z >= 0 && z < c.nz) ? iso::grid_coord(uint32_t(z), uint32_t(c.nz), p.amin[2],
                                                             p.asize[2])
                                           : 0.0f;
        }
        for (int i = tid; i < c.RY; i += BLOCK) {
            int y = c.Y0 - 1 + i;
            s.gy[i] = (y >= 0 && y < c.ny) ? iso::grid_coord(uint32_t(y), uint32_t(c.ny), p.amin[1],
                                                             p.asize[1])
                                           : 0.0f;
        }
        for (int w = tid; w < c.NW; w += BLOCK) {
            s.zval[w] = iso::range_mask(w, zf - c.Z0 + 32, zl - c.Z0 + 32);
            // E cells by high-corner column: cz in [Z0-1, Z1-1] and in the grid.
            s.ecol[w] = iso::range_mask(w, max(32, 33 - c.Z0), min(c.Z1 - 1, c.nz - 2) - c.Z0 + 33);
            // own cells: cz in [Z0-1, Z1-2]
            s.ocell[w] = iso::range_mask(w, max(32, 33 - c.Z0), c.Z1 - c.Z0 + 31);
            // owned points: z in [Z0, Z1)
            s.ocol[w] = iso::range_mask(w, 32, c.Z1 - c.Z0 + 31);
        }
        const int ylo = max(c.Y0 - 1, 0), yhi = min(c.Y1, c.ny - 1);  // loaded rows
        const int hyE0 = max(1, 2 - c.Y0), hyE1 = min(c.Y1 - 1, c.ny - 2) - c.Y0 + 2;
        const int hyO0 = hyE0, hyO1 = c.Y1 - c.Y0;

        // Issue the TMA bulk copies of slab j (plane pfirst + j).
        auto issue = [&](int j) {
            const int pl = pfirst + j;
            const unsigned long long q = qbase + j;
            const int slot = int(q % S);
            uint32_t total = 0;
            for (int ly = 0; ly < c.RY; ++ly) {
                int y = c.Y0 - 1 + ly;
                if (y < ylo || y > yhi) continue;
                long long g = ((long long)pl * c.ny + y) * c.nz + zf;
                int shift = int(g & 3);
                int nfl = (zl - zf + 1) + shift;
                total += uint32_t((nfl + 3) & ~3) * 4u;
            }
            s.gx[slot] = iso::grid_coord(uint32_t(pl), uint32_t(c.nx), p.amin[0], p.asize[0]);
            iso::mbar_expect_tx(&s.bar[slot], total);
            for (int ly = 0; ly < c.RY; ++ly) {
                int y = c.Y0 - 1 + ly;
                if (y < ylo || y > yhi) continue;
                long long g = ((long long)pl * c.ny + y) * c.nz + zf;
                int shift = int(g & 3);
                int nfl = (zl - zf + 1) + shift;
                int shv = (((shift - zf + c.Z0) % 4) + 4) % 4;
                int dst = (zf - c.Z0 + 4) - shift + shv;
                s.sh[slot * c.RY + ly] = shv;
                iso::bulk_g2s(s.vals + size_t(slot * c.RY + ly) * c.CZP + dst, p.vals + (g - shift),
                              uint32_t((nfl + 3) & ~3) * 4u, &s.bar[slot]);
            }
        };

        if (tid == 0) {
            for (int j = 0; j < min(S, nslab); ++j) issue(j);
        }

        for (int j = 0; j < nslab; ++j) {
            const int pl = pfirst + j;
            const unsigned long long q = qbase + j;
            const int slot = int(q % S);
            const uint32_t parity = uint32_t((q / S) & 1ull);
            if (!iso::mbar_wait(&s.bar[slot], parity)) {
                atomicCAS(p.status, 0, int(ISO_ERR_TIMEOUT));
                s_abort = 1;
            }
            __syncthreads();
            if (s_abort) {
                // drain: wait (bounded) for copies still in flight, then leave
                if (tid == 0) {
                    for (int jj = j + 1; jj < min(nslab, j + S); ++jj) {
                        unsigned long long qq = qbase + jj;
                        iso::mbar_wait(&s.bar[qq % S], uint32_t((qq / S) & 1ull));
                    }
                }
                return;
            }
            const int sp = j > 0 ? int((q - 1) % S) : -1;

            // (1) sign bits of the new slab
            for (int wi = warp; wi < RW; wi += NWARP) {
                int ly = wi / c.NW, w = wi % c.NW;
                int y = c.Y0 - 1 + ly;
                bool rv = y >= ylo && y <= yhi;
                bool valid = rv && ((s.zval[w] >> lane) & 1u);
                float v = valid ? valat(s, c, slot, ly, 32 * w + lane) : 0.0f;
                uint32_t b = __ballot_sync(~0u, valid && iso::below(v, c.level));
                if (lane == 0) s.bm[((size_t(slot) * NB + B_SGN) * c.RY + ly) * c.NW + w] = b;
            }
            __syncthreads();

            // (2) crossed and snapped edges whose high endpoint lies in this slab
            for (int i = tid; i < 3 * RW; i += BLOCK) {
                int ax = i / RW, r = i % RW, ly = r / c.NW, w = r % c.NW;
                int y = c.Y0 - 1 + ly;
                bool rv = y >= ylo && y <= yhi;
                const uint32_t* sg = bmrow(s, c, slot, B_SGN, ly);
                uint32_t cr = 0;
                if (rv) {
                    if (ax == 0) {
                        if (sp >= 0) cr = (sg[w] ^ bmrow(s, c, sp, B_SGN, ly)[w]) & s.zval[w];
                    } else if (ax == 1) {
                        if (ly >= 1 && y - 1 >= ylo)
                            cr = (sg[w] ^ bmrow(s, c, slot, B_SGN, ly - 1)[w]) & s.zval[w];
                    } else {
                        cr = (sg[w] ^ prev1(sg, w)) & s.zval[w] & prev1(s.zval, w);
                    }
                }
                uint32_t lo = 0, hi = 0;
                uint32_t bits = cr;
                while (bits) {
                    int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    int col = 32 * w + b;
                    int sa = ax == 0 ? sp : slot;
                    int ra = ax == 1 ? ly - 1 : ly;
                    int ca = ax == 2 ? col - 1 : col;
                    float va = valat(s, c, sa, ra, ca), vb = valat(s, c, slot, ly, col);
                    float ax_ = s.gx[sa], ay = s.gy[ra], az = s.gz[ca];
                    float bx = s.gx[slot], by = s.gy[ly], bz = s.gz[col];
                    float t = iso::cross_t(c.level, va, vb);
                    float px = iso::lerp1(t, ax_, bx), py = iso::lerp1(t, ay, by),
                          pz = iso::lerp1(t, az, bz);
                    if (px == ax_ && py == ay && pz == az) lo |= 1u << b;
                    else if (px == bx && py == by && pz == bz) hi |= 1u << b;
                }
                s.bm[((size_t(slot) * NB + B_CRX + ax) * c.RY + ly) * c.NW + w] = cr;
                s.bm[((size_t(slot) * NB + B_LOX + ax) * c.RY + ly) * c.NW + w] = lo;
                s.bm[((size_t(slot) * NB + B_HIX + ax) * c.RY + ly) * c.NW + w] = hi;
            }
            __syncthreads();

            // Tiles ready after this slab: P = pl - 1 (needs pl) and, at the
            // last plane of the grid, P = pl itself.
            for (int pass = 0; pass < 2; ++pass) {
                const int P = pass == 0 ? pl - 1 : pl;
                if (pass == 1 && pl != c.nx - 1) break;
                if (P < Pa || P >= Pb) continue;
                c.P = P;
                c.sB = int((qbase + (P - pfirst)) % S);
                c.sA = P >= 1 ? int((qbase + (P - 1 - pfirst)) % S) : -1;
                c.sC = P + 1 <= c.nx - 1 ? int((qbase + (P + 1 - pfirst)) % S) : -1;
                const bool L0 = P >= 1, L1 = P + 1 <= c.nx - 1;

                // T1: cell masks of both layers; clear detailed marks
                for (int i = tid; i < 2 * RW; i += BLOCK) {
                    int L = i / RW, r = i % RW, hy = r / c.NW, hw = r % c.NW;
                    uint32_t act = 0, fre = 0, snp = 0;
                    bool lok = L ? L1 : L0;
                    if (lok && hy >= hyE0 && hy <= hyE1 && hw >= 1) {
                        uint32_t em = s.ecol[hw];
                        if (em) {
                            int lo = L ? c.sB : c.sA, hi = L ? c.sC : c.sB;
                            const uint32_t* a0 = bmrow(s, c, lo, B_SGN, hy - 1);
                            const uint32_t* a1 = bmrow(s, c, lo, B_SGN, hy);
                            const uint32_t* b0 = bmrow(s, c, hi, B_SGN, hy - 1);
                            const uint32_t* b1 = bmrow(s, c, hi, B_SGN, hy);
                            uint32_t w0 = a0[hw], w1 = prev1(a0, hw), w2 = a1[hw], w3 = prev1(a1, hw);
                            uint32_t w4 = b0[hw], w5 = prev1(b0, hw), w6 = b1[hw], w7 = prev1(b1, hw);
                            uint32_t and8 = w0 & w1 & w2 & w3 & w4 & w5 & w6 & w7;
                            uint32_t or8 = w0 | w1 | w2 | w3 | w4 | w5 | w6 | w7;
                            act = (or8 & ~and8) & em;
                            if (act) {
                                uint32_t sn = 0;
                                // x edges (stored in the high plane) at rows hy-1, hy; cols c-1, c
                                for (int rr = hy - 1; rr <= hy; ++rr) {
                                    const uint32_t* xl = bmrow(s, c, hi, B_LOX, rr);
                                    const uint32_t* xh = bmrow(s, c, hi, B_HIX, rr);
                                    sn |= xl[hw] | prev1(xl, hw) | xh[hw] | prev1(xh, hw);
                                }
                                // y edges in both planes at row hy; cols c-1, c
                                for (int pp = 0; pp < 2; ++pp) {
                                    int pls = pp ? hi : lo;
                                    const uint32_t* yl = bmrow(s, c, pls, B_LOY, hy);
                                    const uint32_t* yh = bmrow(s, c, pls, B_HIY, hy);
                                    sn |= yl[hw] | prev1(yl, hw) | yh[hw] | prev1(yh, hw);
                                    // z edges in both planes at rows hy-1, hy; col c
                                    for (int rr = hy - 1; rr <= hy; ++rr) {
                                        sn |= bmrow(s, c, pls, B_LOZ, rr)[hw] |
                                              bmrow(s, c, pls, B_HIZ, rr)[hw];
                                    }
                                }
                                snp = act & sn;
                                fre = act & ~sn;
                            }
                        }
                    }
                    s.act[i] = act;
                    s.fre[i] = fre;
                    s.snp[i] = snp;
                }
                for (int i = tid; i < 4 * RW; i += BLOCK) s.du[i] = 0;
                __syncthreads();

                // T2: own face counts; detailed handling of cells with snapped edges
                for (int i = tid; i < 2 * RW; i += BLOCK) {
                    int L = i / RW, r = i % RW, hy = r / c.NW, hw = r % c.NW;
                    uint32_t act = s.act[i];
                    uint32_t own = (L == 0 && hy >= hyO0 && hy <= hyO1) ? (act & s.ocell[hw]) : 0u;
                    uint32_t snp = s.snp[i];
                    uint32_t faces = 0;
                    uint32_t bits = own | snp;
                    while (bits) {
                        int b = __ffs(bits) - 1;
                        bits &= bits - 1;
                        int hc = 32 * hw + b;
                        uint32_t cs = cell_case(s, c, L, hy, hc);
                        uint32_t nt;
                        if ((snp >> b) & 1u) {
                            uint32_t key[12];
                            cell_keys(s, c, L, hy, hc, s.estat[cs], key);
                            const int8_t* tr = s.tri + cs * 15;
                            nt = 0;
                            for (int k = 0; k < 15 && tr[k] >= 0; k += 3) {
                                uint32_t k0 = key[tr[k]], k1 = key[tr[k + 1]], k2 = key[tr[k + 2]];
                                if (k0 == k1 || k0 == k2 || k1 == k2) continue;
                                ++nt;
                                uint32_t kk[3] = {k0, k1, k2};
#pragma unroll
                                for (int m = 0; m < 3; ++m) {
                                    int rel, row, colk, type;
                                    key_split(c, kk[m], rel, row, colk, type);
                                    if (key_owned(c, rel, row, colk))
                                        atomicOr(&s.du[(type * c.RY + row) * c.NW + (colk >> 5)],
                                                 1u << (colk & 31));
                                }
                            }
                        } else {
                            nt = s.ntri[cs];
                        }
                        if ((own >> b) & 1u) faces += nt;
                    }
                    if (L == 0) s.fcnt[r] = faces;
                }
                __syncthreads();

                // T3: vertex existence for the owned points (plane P)
                for (int i = tid; i < RW; i += BLOCK) {
                    int ly = i / c.NW, w = i % c.NW;
                    uint32_t e0 = 0, e1 = 0, e2 = 0, e3 = 0;
                    uint32_t om = (ly >= 1 && ly <= c.Y1 - c.Y0) ? s.ocol[w] : 0u;
                    if (om) {
                        const uint32_t* f0a = s.fre + ly * c.NW;
                        const uint32_t* f0b = s.fre + (ly + 1) * c.NW;
                        const uint32_t* f1a = s.fre + RW + ly * c.NW;
                        const uint32_t* f1b = s.fre + RW + (ly + 1) * c.NW;
                        uint32_t g0 = f0a[w], g0n = next1(f0a, w, c.NW), g1 = f0b[w],
                                 g1n = next1(f0b, w, c.NW);
                        uint32_t h0 = f1a[w], h0n = next1(f1a, w, c.NW), h1 = f1b[w];
                        const int sB = c.sB;
                        uint32_t cr, sn;
                        cr = bmrow(s, c, sB, B_CRX, ly)[w];
                        sn = bmrow(s, c, sB, B_LOX, ly)[w] | bmrow(s, c, sB, B_HIX, ly)[w];
                        e0 = cr & ~sn & ((g0 | g0n | g1 | g1n) | s.du[(0 * c.RY + ly) * c.NW + w]) & om;
                        cr = bmrow(s, c, sB, B_CRY, ly)[w];
                        sn = bmrow(s, c, sB, B_LOY, ly)[w] | bmrow(s, c, sB, B_HIY, ly)[w];
                        e1 = cr & ~sn & ((g0 | g0n | h0 | h0n) | s.du[(1 * c.RY + ly) * c.NW + w]) & om;
                        cr = bmrow(s, c, sB, B_CRZ, ly)[w];
                        sn = bmrow(s, c, sB, B_LOZ, ly)[w] | bmrow(s, c, sB, B_HIZ, ly)[w];
                        e2 = cr & ~sn & ((g0 | g1 | h0 | h1) | s.du[(2 * c.RY + ly) * c.NW + w]) & om;
                        e3 = s.du[(3 * c.RY + ly) * c.NW + w] & om;
                    }
                    s.ex[0 * RW + i] = e0;
                    s.ex[1 * RW + i] = e1;
                    s.ex[2 * RW + i] = e2;
                    s.ex[3 * RW + i] = e3;
                    s.vcnt[i] = __popc(e0) + __popc(e1) + __popc(e2) + __popc(e3);
                }
                __syncthreads();

                // T4: offsets
                uint32_t VT, FT;
                scan2<BLOCK>(s.vcnt, s.fcnt, RW, scan_tmp, VT, FT);
                const long long tile = ((long long)P * c.nRT + c.rt) * c.nZT + c.zt;
                if (tid == 0) {
                    unsigned long long vo = 0, fo = 0;
                    if (VT) vo = atomicAdd(&p.ctr[1], (unsigned long long)VT);
                    if (FT) fo = atomicAdd(&p.ctr[2], (unsigned long long)FT);
                    s.misc[1] = vo;
                    s.misc[2] = fo;
                    McTileRec rec;
                    rec.vOff = uint32_t(vo);
                    rec.vCnt = VT;
                    rec.fOff = uint32_t(fo);
                    rec.fCnt = FT;
                    p.rec[tile] = rec;
                }
                __syncthreads();
                const unsigned long long vOff = s.misc[1], fOff = s.misc[2];
                const bool vfit = vOff + VT <= (unsigned long long)p.capSV;
                const bool ffit = fOff + FT <= (unsigned long long)p.capSF;

                // T5a: staged vertices, in key order
                if (VT && vfit) {
                    for (int i = tid; i < RW; i += BLOCK) {
                        uint32_t e[4] = {s.ex[i], s.ex[RW + i], s.ex[2 * RW + i], s.ex[3 * RW + i]};
                        uint32_t any = e[0] | e[1] | e[2] | e[3];
                        if (!any) continue;
                        int ly = i / c.NW, w = i % c.NW;
                        unsigned long long o = vOff + s.vcnt[i];
                        const int sB = c.sB;
                        while (any) {
                            int b = __ffs(any) - 1;
                            any &= any - 1;
                            int col = 32 * w + b;
#pragma unroll
                            for (int type = 0; type < 4; ++type) {
                                if (!((e[type] >> b) & 1u)) continue;
                                float x, y, z;
                                float bx = s.gx[sB], by = s.gy[ly], bz = s.gz[col];
                                if (type == 3) {
                                    x = bx; y = by; z = bz;
                                } else {
                                    int sa = type == 0 ? c.sA : sB;
                                    int ra = type == 1 ? ly - 1 : ly;
                                    int ca = type == 2 ? col - 1 : col;
                                    float va = valat(s, c, sa, ra, ca), vb = valat(s, c, sB, ly, col);
                                    float t = iso::cross_t(c.level, va, vb);
                                    x = iso::lerp1(t, s.gx[sa], bx);
                                    y = iso::lerp1(t, s.gy[ra], by);
                                    z = iso::lerp1(t, s.gz[ca], bz);
                                }
                                uint32_t key = (uint32_t((ly - 1) * c.ZC + (col - 32)) << 2) | type;
                                p.sv[o++] = make_float4(x, y, z, __uint_as_float(key));
                            }
                        }
                    }
                }
                // T5b: staged faces of own cells, in cell order
                if (FT && ffit) {
                    for (int i = tid; i < RW; i += BLOCK) {
                        int hy = i / c.NW, hw = i % c.NW;
                        if (hy < hyO0 || hy > hyO1 || hw < 1) continue;
                        uint32_t own = s.act[i] & s.ocell[hw];
                        if (!own) continue;
                        uint32_t snp = s.snp[i];
                        unsigned long long o = fOff + s.fcnt[i];
                        while (own) {
                            int b = __ffs(own) - 1;
                            own &= own - 1;
                            int hc = 32 * hw + b;
                            uint32_t cs = cell_case(s, c, 0, hy, hc);
                            uint32_t key[12];
                            cell_keys(s, c, 0, hy, hc, s.estat[cs], key);
                            const bool check = (snp >> b) & 1u;
                            const int8_t* tr = s.tri + cs * 15;
                            for (int k = 0; k < 15 && tr[k] >= 0; k += 3) {
                                uint32_t k0 = key[tr[k]], k1 = key[tr[k + 1]], k2 = key[tr[k + 2]];
                                if (check && (k0 == k1 || k0 == k2 || k1 == k2)) continue;
                                uint32_t* dst = p.sf + 3 * o++;
                                dst[0] = key_ref(c, k0);
                                dst[1] = key_ref(c, k1);
                                dst[2] = key_ref(c, k2);
                            }
                        }
                    }
                }
                __syncthreads();
            }

            // Tile pl - 1 was the last user of slab pl - 2: reuse its slot.
            if (tid == 0 && j >= 2 && j - 2 + S < nslab) issue(j - 2 + S);
        }
        qbase += nslab;
        __syncthreads();
    }
}

// Exclusive prefix of per-tile counts (one CTA).
__global__ void __launch_bounds__(1024) mc_tile_scan(const McTileRec* __restrict__ rec, uint2* pre,
                                                     long long n, long long* counts, int* status,
                                                     long long capV, long long capF) {
    __shared__ unsigned long long wa[32], wb[32];
    __shared__ unsigned long long carry[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) { carry[0] = 0; carry[1] = 0; }
    __syncthreads();
    for (long long base = 0; base < n; base += 1024) {
        long long i = base + tid;
        unsigned long long a = 0, b = 0;
        if (i < n) { McTileRec r = rec[i]; a = r.vCnt; b = r.fCnt; }
        unsigned long long ia = a, ib = b;
        for (int d = 1; d < 32; d <<= 1) {
            unsigned long long xa = __shfl_up_sync(~0u, ia, d), xb = __shfl_up_sync(~0u, ib, d);
            if (lane >= d) { ia += xa; ib += xb; }
        }
        if (lane == 31) { wa[warp] = ia; wb[warp] = ib; }
        __syncthreads();
        if (warp == 0) {
            unsigned long long va = wa[lane], vb = wb[lane];
            for (int d = 1; d < 32; d <<= 1) {
                unsigned long long xa = __shfl_up_sync(~0u, va, d), xb = __shfl_up_sync(~0u, vb, d);
                if (lane >= d) { va += xa; vb += xb; }
            }
            wa[lane] = va;
            wb[lane] = vb;
        }
        __syncthreads();
        unsigned long long ea = carry[0] + (warp ? wa[warp - 1] : 0ull) + ia - a;
        unsigned long long eb = carry[1] + (warp ? wb[warp - 1] : 0ull) + ib - b;
        if (i < n) pre[i] = make_uint2(uint32_t(ea), uint32_t(eb));
        __syncthreads();
        if (tid == 0) { carry[0] += wa[31]; carry[1] += wb[31]; }
        __syncthreads();
    }
    if (tid == 0) {
        counts[0] = (long long)carry[0];
        counts[1] = (long long)carry[1];
        if ((long long)carry[0] > capV || (long long)carry[1] > capF)
            atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
    }
}

// Final vertices and faces of one tile.
constexpr int RES_BLOCK = 128;
constexpr int RES_KCAP = 2048;

__global__ void __launch_bounds__(RES_BLOCK) mc_resolve(const McParams p) {
    const McTiles& T = p.t;
    const long long tile = blockIdx.x;
    const McTileRec rec = p.rec[tile];
    if (rec.vCnt == 0 && rec.fCnt == 0) return;
    const uint2 pre = p.pre[tile];
    const int tid = threadIdx.x;
    const bool vfit = (unsigned long long)rec.vOff + rec.vCnt <= (unsigned long long)p.capSV;
    const bool ffit = (unsigned long long)rec.fOff + rec.fCnt <= (unsigned long long)p.capSF;
    for (uint32_t i = tid; i < rec.vCnt && vfit; i += RES_BLOCK) {
        long long o = (long long)pre.x + i;
        if (o >= p.capV) break;
        float4 v = p.sv[rec.vOff + i];
        p.vout[3 * o + 0] = v.x;
        p.vout[3 * o + 1] = v.y;
        p.vout[3 * o + 2] = v.z;
    }
    if (rec.fCnt == 0 || !ffit) return;

    // Stage the key lists of the tiles faces may refer to (slot bits: plane,
    // row group, z chunk one step back).
    __shared__ uint32_t keys[RES_KCAP];
    __shared__ uint32_t segOff[8], segLen[8], segBase[8], segVOff[8];
    __shared__ int useGlobal;
    const int zt = int(tile % T.nZT);
    const int rt = int((tile / T.nZT) % T.nRT);
    const int P = int(tile / ((long long)T.nZT * T.nRT));
    if (tid == 0) {
        uint32_t tot = 0;
        for (int sl = 0; sl < 8; ++sl) {
            int pp = P - (sl >> 2), rr = rt - ((sl >> 1) & 1), zz = zt - (sl & 1);
            segOff[sl] = tot;
            segLen[sl] = 0;
            segBase[sl] = 0;
            segVOff[sl] = 0;
            if (pp < 0 || rr < 0 || zz < 0) continue;
            long long t2 = ((long long)pp * T.nRT + rr) * T.nZT + zz;
            McTileRec r2 = p.rec[t2];
            // a neighbour whose staging did not fit has no keys to search (the
            // scan already flagged the overflow; the caller retries)
            if ((unsigned long long)r2.vOff + r2.vCnt > (unsigned long long)p.capSV) continue;
            segLen[sl] = r2.vCnt;
            segBase[sl] = p.pre[t2].x;
            segVOff[sl] = r2.vOff;
            tot += r2.vCnt;
        }
        useGlobal = tot > RES_KCAP;
    }
    __syncthreads();
    if (!useGlobal) {
        for (int sl = 0; sl < 8; ++sl) {
            for (uint32_t i = tid; i < segLen[sl]; i += RES_BLOCK)
                keys[segOff[sl] + i] = __float_as_uint(p.sv[segVOff[sl] + i].w);
        }
    }
    __syncthreads();
    for (uint32_t f = tid; f < rec.fCnt; f += RES_BLOCK) {
        long long o = (long long)pre.y + f;
        if (o >= p.capF) break;
        const uint32_t* src = p.sf + 3ull * (rec.fOff + f);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            uint32_t ref = src[m];
            uint32_t sl = ref >> 24, local = ref & 0xffffffu;
            uint32_t lo = 0, hi = segLen[sl];
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                uint32_t k = useGlobal ? __float_as_uint(p.sv[segVOff[sl] + mid].w)
                                       : keys[segOff[sl] + mid];
                if (k < local) lo = mid + 1; else hi = mid;
            }
            uint32_t k = lo < segLen[sl] ? (useGlobal ? __float_as_uint(p.sv[segVOff[sl] + lo].w)
                                                      : keys[segOff[sl] + lo])
                                         : 0xffffffffu;
            int idx;
            if (k == local) {
                idx = int(segBase[sl] + lo);
            } else {
                atomicCAS(p.status, 0, int(ISO_ERR_LOOKUP));
                idx = -1;
            }
            p.fout[3 * o + m] = idx;
        }
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
    long long grid = (long long)sms * per;
    if (grid > p.t.nItems) grid = p.t.nItems;
    if (grid < 1) grid = 1;
    k<<<unsigned(grid), BLOCK, p.t.smemBytes, st>>>(p);
    return cudaGetLastError() == cudaSuccess ? 0 : ISO_ERR_CUDA;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host API

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
    const size_t budget = size_t(optin) - 2048;
    // Full-z tiles when they fit with at least one row; else z chunks of one row.
    int R = std::max(1, rows);
    int ZC = (nz + 31) / 32 * 32;
    if (zchunk > 0 && zchunk < ZC) ZC = std::max(32, zchunk / 32 * 32);
    auto fits = [&](int r, int zc) {
        McTiles u = t;
        u.R = r; u.ZC = zc; u.RY = r + 2; u.NW = zc / 32 + 2; u.CZP = zc + 12;
        return make_layout(u).total <= budget;
    };
    while (R > 1 && !fits(R, ZC)) --R;
    if (!fits(R, ZC)) {
        R = 1;
        while (ZC > 32 && !fits(1, ZC)) ZC -= 32;
        if (!fits(1, ZC)) return ISO_ERR_ARG;
    }
    if (ZC < nz) R = 1;  // split z => one row per tile keeps tiles contiguous
    t.R = R; t.ZC = ZC;
    t.RY = R + 2; t.NW = ZC / 32 + 2; t.CZP = ZC + 12;
    t.nRT = (ny + R - 1) / R;
    t.nZT = (nz + ZC - 1) / ZC;
    t.nTiles = (long long)nx * t.nRT * t.nZT;
    if ((long long)R * ZC * 4 >= (1ll << 24)) return ISO_ERR_ARG;
    const Layout L = make_layout(t);
    t.smemBytes = L.total;
    t.ctasPerSm = std::max(1, int((size_t(228) * 1024) / (L.total + 1024)));
    if (t.ctasPerSm > 8) t.ctasPerSm = 8;
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

size_t mc_workspace_bytes(const McTiles& t, long long capV, long long capF) {
    size_t o = 0;
    o = al16(o + size_t(t.nTiles) * sizeof(McTileRec));
    o = al16(o + size_t(t.nTiles) * sizeof(uint2));
    o = al16(o + size_t(std::max<long long>(capV, 1)) * sizeof(float4));
    o = al16(o + size_t(std::max<long long>(capF, 1)) * 3 * sizeof(uint32_t));
    o = al16(o + 4 * sizeof(unsigned long long));
    return o + 256;
}

int mc_launch(const McParams& p0, void* ws, size_t ws_bytes, cudaStream_t st) {
    McParams p = p0;
    const McTiles& t = p.t;
    const size_t need = mc_workspace_bytes(t, p.capV, p.capF);
    if (ws_bytes < need) return ISO_ERR_WORKSPACE;
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    p.rec = reinterpret_cast<McTileRec*>(b + o); o = al16(o + size_t(t.nTiles) * sizeof(McTileRec));
    p.pre = reinterpret_cast<uint2*>(b + o);     o = al16(o + size_t(t.nTiles) * sizeof(uint2));
    p.sv = reinterpret_cast<float4*>(b + o);     o = al16(o + size_t(std::max<long long>(p.capV, 1)) * sizeof(float4));
    p.sf = reinterpret_cast<uint32_t*>(b + o);   o = al16(o + size_t(std::max<long long>(p.capF, 1)) * 3 * sizeof(uint32_t));
    p.ctr = reinterpret_cast<unsigned long long*>(b + o);
    p.capSV = p.capV;
    p.capSF = p.capF;
    if (cudaMemsetAsync(p.ctr, 0, 4 * sizeof(unsigned long long), st) != cudaSuccess)
        return ISO_ERR_CUDA;
    int rc = t.threads == 512 ? launch_extract<512>(p, st) : launch_extract<256>(p, st);
    if (rc) return rc;
    mc_tile_scan<<<1, 1024, 0, st>>>(p.rec, p.pre, t.nTiles, p.counts, p.status, p.capV, p.capF);
    if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    if (t.nTiles > 0x7fffffffll) return ISO_ERR_ARG;
    mc_resolve<<<unsigned(t.nTiles), RES_BLOCK, 0, st>>>(p);
    if (cudaGetLastError() != cudaSuccess) return ISO_ERR_CUDA;
    return 0;
}
