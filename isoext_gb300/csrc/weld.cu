// Exact-position weld of a point list with device-side sizes (isoext
// src/utils.cu:32-59: vertices with equal positions become one), for the
// one-call sparse marching cubes.  The output numbers the distinct positions in
// the order of their first entry in the list, and every triangle index names
// the first entry with its position.
//
//   weld_insert   hash table of positions: a slot keeps the smallest entry
//                 with its position.  Two entries per thread, their probes in
//                 flight together (the kernel is bound by the latency of
//                 dependent atomics and gathers, not by bytes).
//   weld_number   per tile of 512 entries: each entry's first entry (table
//                 lookup), the tile's number of first entries, the exclusive
//                 prefix over tiles by decoupled look-back, and the first
//                 entries' new numbers and positions written out.
//   weld_remap    triangle indices -> new numbers.
#include <algorithm>
#include <cstdint>

#include <cub/device/device_scan.cuh>

#include "common.cuh"
#include "lookback.cuh"
#include "profile.cuh"

namespace {

constexpr int WELD_THREADS = 256;
constexpr int WELD_PER = 2;                           // entries per thread (insert, numbering)
constexpr int WELD_TILE = WELD_THREADS * WELD_PER;    // entries per CTA
constexpr int REMAP_PER = 4;                          // triangle indices per thread of the remap
constexpr uint32_t WELD_EMPTY = 0xffffffffu;          // a free table slot
constexpr uint32_t WELD_NEW = 0x80000000u;            // rep[a]: a is a first entry; low bits its new number
constexpr uint32_t WELD_PROBES = 512;  // the table is at most half full when the capacity holds the positions

using iso::pos_bits;
using iso::pos_hash;

struct Key {
    uint32_t x, y, z;
};

__device__ __forceinline__ Key key_of(const float* __restrict__ pts, long long a) {
    return Key{pos_bits(pts[3 * a]), pos_bits(pts[3 * a + 1]), pos_bits(pts[3 * a + 2])};
}
__device__ __forceinline__ bool same(const Key& a, const Key& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ uint32_t slot_of(const Key& k, uint32_t mask) { return pos_hash(k.x, k.y, k.z) & mask; }

// The rest of an insert whose first probe met another position.
__device__ __noinline__ void insert_probe(const float* __restrict__ pts, uint32_t* table, uint32_t mask, Key k,
                                          uint32_t h, uint32_t a, int* status) {
    if (*(volatile int*)status == int(ISO_ERR_OVERFLOW)) return;  // the output is discarded anyway
    for (uint32_t p = 1; p <= mask && p < WELD_PROBES; ++p) {
        h = (h + 1) & mask;
        const uint32_t cur = atomicCAS(&table[h], WELD_EMPTY, a);
        if (cur == WELD_EMPTY) return;
        if (same(key_of(pts, cur), k)) {
            if (a < cur) atomicMin(&table[h], a);
            return;
        }
    }
    atomicCAS(status, 0, int(ISO_ERR_OVERFLOW));
}

// The rest of a lookup whose first probe met another position.
__device__ __noinline__ uint32_t lookup_probe(const float* __restrict__ pts, const uint32_t* table, uint32_t mask,
                                              Key k, uint32_t h, uint32_t a) {
    for (uint32_t p = 1; p <= mask && p < WELD_PROBES; ++p) {
        h = (h + 1) & mask;
        const uint32_t cur = table[h];
        if (cur == WELD_EMPTY) break;
        if (same(key_of(pts, cur), k)) return cur;
    }
    return a;  // not placed (the status says overflow)
}

__global__ void __launch_bounds__(WELD_THREADS) weld_insert(const float* __restrict__ pts, long long A,
                                                            uint32_t* table, uint32_t mask, int* status,
                                                            const long long* __restrict__ dn) {
    if (dn) A = dn[0];
    const long long base = (long long)blockIdx.x * WELD_TILE + threadIdx.x;
    Key k[WELD_PER];
    uint32_t h[WELD_PER], cur[WELD_PER];
    bool live[WELD_PER];
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e) {
        const long long a = base + e * WELD_THREADS;
        live[e] = a < A;
        if (live[e]) k[e] = key_of(pts, a);
    }
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e)
        if (live[e]) {
            h[e] = slot_of(k[e], mask);
            cur[e] = atomicCAS(&table[h[e]], WELD_EMPTY, uint32_t(base + e * WELD_THREADS));
        }
    Key o[WELD_PER];
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e)
        if (live[e] && cur[e] != WELD_EMPTY) o[e] = key_of(pts, cur[e]);
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e) {
        if (!live[e] || cur[e] == WELD_EMPTY) continue;
        const uint32_t a = uint32_t(base + e * WELD_THREADS);
        if (same(o[e], k[e])) {
            if (a < cur[e]) atomicMin(&table[h[e]], a);
        } else {
            insert_probe(pts, table, mask, k[e], h[e], a, status);
        }
    }
}

// rep[a] <- WELD_NEW | new number for a first entry, else the first entry with
// a's position; vout / vsrc <- the first
// entries' positions and entries (up to capV); vtot[0] <- the number of
// distinct positions.  Tiles are taken in ticket order (ctr) and chained by
// look-back (state, one word per tile, zeroed by the caller).
__global__ void __launch_bounds__(WELD_THREADS) weld_number(const float* __restrict__ pts, long long A,
                                                            const uint32_t* __restrict__ table, uint32_t mask,
                                                            uint32_t* __restrict__ rep, unsigned long long* state,
                                                            unsigned int* ctr, float* __restrict__ vout,
                                                            uint32_t* __restrict__ vsrc, long long* vtot, int* status,
                                                            const long long* __restrict__ dn) {
    __shared__ uint32_t tile_s;
    __shared__ uint32_t wsum[WELD_THREADS / 32];
    __shared__ unsigned long long pre_s;
    long long capV = 0x7fffffffll;
    if (dn) {
        A = dn[0];
        capV = dn[3];
    }
    if (threadIdx.x == 0) tile_s = atomicAdd(ctr, 1u);
    __syncthreads();
    const uint32_t tile = tile_s;
    const long long ntile = (A + WELD_TILE - 1) / WELD_TILE;
    if ((long long)tile >= ntile) {
        if (tile == 0 && threadIdx.x == 0) { vtot[0] = 0; vtot[1] = 0; }  // no points
        return;
    }
    // entries a0 .. a0 + 3 of this thread (consecutive: the prefix is in list order)
    const long long a0 = (long long)tile * WELD_TILE + threadIdx.x * WELD_PER;
    Key k[WELD_PER];
    uint32_t h[WELD_PER], cur[WELD_PER], r[WELD_PER];
    bool live[WELD_PER];
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e) {
        live[e] = a0 + e < A;
        r[e] = WELD_EMPTY;
        if (live[e]) k[e] = key_of(pts, a0 + e);
    }
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e)
        if (live[e]) {
            h[e] = slot_of(k[e], mask);
            cur[e] = table[h[e]];
        }
    Key o[WELD_PER];
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e)
        if (live[e] && cur[e] != WELD_EMPTY) o[e] = key_of(pts, cur[e]);
    uint32_t cnt = 0;
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e) {
        if (!live[e]) continue;
        const uint32_t a = uint32_t(a0 + e);
        if (cur[e] != WELD_EMPTY && same(o[e], k[e])) r[e] = cur[e];
        else r[e] = cur[e] == WELD_EMPTY ? a : lookup_probe(pts, table, mask, k[e], h[e], a);
        cnt += r[e] == a ? 1u : 0u;
    }
    // exclusive prefix of first entries: in the tile, then over tiles
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(~0u, inc, d);
        if (lane >= d) inc += v;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < WELD_THREADS / 32; ++w) {
        before += w < warp ? wsum[w] : 0u;
        total += wsum[w];
    }
    if (warp == 0) {
        unsigned long long pv = 0, unused = 0;
        lb_tile(state, tile, total, 0, pv, unused, status);
        if (lane == 0) {
            pre_s = pv;
            if ((long long)tile == ntile - 1) {
                vtot[0] = (long long)(pv + total);
                vtot[1] = 0;
            }
        }
    }
    __syncthreads();
    unsigned long long no = pre_s + before + inc - cnt;
#pragma unroll
    for (int e = 0; e < WELD_PER; ++e) {
        if (a0 + e >= A) break;
        const uint32_t a = uint32_t(a0 + e);
        if (r[e] == a) {
            rep[a] = WELD_NEW | uint32_t(no);
            if ((long long)no < capV) {  // past the capacity the caller sees V and retries
                float* v = vout + 3 * no;
                v[0] = pts[3ll * a]; v[1] = pts[3ll * a + 1]; v[2] = pts[3ll * a + 2];
                if (vsrc) vsrc[no] = a;
            }
            ++no;
        } else {
            rep[a] = r[e];
        }
    }
}

// fout[i] <- the new number of triangle index tri[i]'s position.
__global__ void __launch_bounds__(WELD_THREADS) weld_remap(const int32_t* __restrict__ tri, long long n,
                                                           const uint32_t* __restrict__ rep, int32_t* fout,
                                                           const long long* __restrict__ dn) {
    if (dn) n = dn[2];
    const long long base = (long long)blockIdx.x * (WELD_THREADS * REMAP_PER) + threadIdx.x;
    uint32_t r[REMAP_PER];
#pragma unroll
    for (int e = 0; e < REMAP_PER; ++e) {
        const long long i = base + e * WELD_THREADS;
        r[e] = i < n ? rep[tri ? tri[i] : int32_t(i)] : WELD_NEW;
    }
#pragma unroll
    for (int e = 0; e < REMAP_PER; ++e)
        if (!(r[e] & WELD_NEW)) r[e] = rep[r[e]];  // the first entry with the position: numbered
#pragma unroll
    for (int e = 0; e < REMAP_PER; ++e) {
        const long long i = base + e * WELD_THREADS;
        if (i < n) fout[i] = int32_t(r[e] & ~WELD_NEW);
    }
}

unsigned tiles_for(long long n) { return unsigned(std::max<long long>((n + WELD_TILE - 1) / WELD_TILE, 1)); }

struct WeldDev {
    uint32_t *rep, *table;
    unsigned long long* state;  // look-back words, then the ticket counter
    uint32_t hcap;
    size_t state_bytes, total;
};

WeldDev weld_dev_carve(void* ws, long long capA, long long capU) {
    WeldDev w{};
    const long long u = capU > 0 && capU < capA ? capU : capA;  // distinct positions the table must hold
    w.hcap = 1024;
    while ((long long)w.hcap < 2 * u + 1024) w.hcap <<= 1;
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = ws ? b + o : nullptr;
        o = (o + std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        return p;
    };
    w.rep = reinterpret_cast<uint32_t*>(take(size_t(capA) * 4));
    w.table = reinterpret_cast<uint32_t*>(take(size_t(w.hcap) * 4));
    w.state_bytes = (size_t(tiles_for(capA)) + 1) * 8;
    w.state = reinterpret_cast<unsigned long long*>(take(w.state_bytes));
    w.total = o + 256;
    return w;
}

}  // namespace

size_t weld_dev_workspace(long long capA, long long capU) { return weld_dev_carve(nullptr, capA, capU).total; }

// The weld of eff[0] points (at most capA) whose distinct positions fit capU:
// eff[2] triangle indices (tri == nullptr: index i is point i; at most capT),
// eff[3] vertex capacity of vout.  vtot[0] <- V.
void weld_dev_launch(const float* pts, long long capA, long long capU, const int32_t* tri, long long capT,
                     const long long* eff, void* ws, float* vout, int32_t* fout, long long* vtot, int* status,
                     cudaStream_t st, uint32_t* vsrc) {
    const WeldDev w = weld_dev_carve(ws, capA, capU);
    iso::ProfScope ps("dc_weld", st, (capT > 0 ? 1 : 0) + (capA > 0 ? 2 : 0));
    if (capA > 0) {
        const unsigned tiles = tiles_for(capA);
        unsigned int* ctr = reinterpret_cast<unsigned int*>(w.state + tiles);
        cudaMemsetAsync(w.table, 0xff, size_t(w.hcap) * 4, st);
        cudaMemsetAsync(w.state, 0, w.state_bytes, st);
        weld_insert<<<tiles, WELD_THREADS, 0, st>>>(pts, capA, w.table, w.hcap - 1, status, eff);
        weld_number<<<tiles, WELD_THREADS, 0, st>>>(pts, capA, w.table, w.hcap - 1, w.rep, w.state, ctr, vout, vsrc,
                                                    vtot, status, eff);
    } else {
        cudaMemsetAsync(vtot, 0, 16, st);
    }
    if (capT > 0) {
        const long long per = (long long)WELD_THREADS * REMAP_PER;
        weld_remap<<<unsigned(std::max<long long>((capT + per - 1) / per, 1)), WELD_THREADS, 0, st>>>(tri, capT,
                                                                                                     w.rep, fout, eff);
    }
}

// ---------------------------------------------------------------------------
// Exact-position weld of a mesh (isoext src/utils.cu:32-59 with the degenerate
// test of src/mc/nagae.cu:71): vertices with equal positions merge into the
// first of them, faces with two equal vertices are dropped, and vertices no
// remaining face uses are dropped.  The survivors keep their order (first
// occurrence).  The marching cubes of a grid whose spacing comes within a few
// ulps of its coordinates needs it: there, vertices of distinct grid edges can
// round to one position.

namespace {

__global__ void __launch_bounds__(WELD_THREADS) mesh_lookup(const float* __restrict__ pts, long long V,
                                                            const uint32_t* __restrict__ table, uint32_t mask,
                                                            uint32_t* __restrict__ rep) {
    const long long a = (long long)blockIdx.x * WELD_THREADS + threadIdx.x;
    if (a >= V) return;
    const Key k = key_of(pts, a);
    uint32_t h = slot_of(k, mask);
    const uint32_t cur = table[h];
    if (cur != WELD_EMPTY && same(key_of(pts, cur), k)) rep[a] = cur;
    else rep[a] = cur == WELD_EMPTY ? uint32_t(a) : lookup_probe(pts, table, mask, k, h, uint32_t(a));
}

// Faces through rep; keep[i] = no two corners at one position; used[v] = 1
// for the corners of kept faces (stores of one value: the races are benign).
__global__ void __launch_bounds__(WELD_THREADS) mesh_faces(const int32_t* __restrict__ f, long long F,
                                                           const uint32_t* __restrict__ rep,
                                                           uint32_t* __restrict__ f2, uint32_t* __restrict__ keep,
                                                           uint32_t* __restrict__ used) {
    const long long i = (long long)blockIdx.x * WELD_THREADS + threadIdx.x;
    if (i >= F) return;
    const uint32_t a = rep[f[3 * i]], b = rep[f[3 * i + 1]], c = rep[f[3 * i + 2]];
    const bool k = a != b && a != c && b != c;
    keep[i] = k ? 1u : 0u;
    f2[3 * i] = a; f2[3 * i + 1] = b; f2[3 * i + 2] = c;
    if (k) { used[a] = 1u; used[b] = 1u; used[c] = 1u; }
}

__global__ void __launch_bounds__(WELD_THREADS) mesh_write(const float* __restrict__ v, long long V, long long F,
                                                           const uint32_t* __restrict__ used,
                                                           const uint32_t* __restrict__ vnum,
                                                           const uint32_t* __restrict__ keep,
                                                           const uint32_t* __restrict__ fnum,
                                                           const uint32_t* __restrict__ f2, float* __restrict__ vout,
                                                           int32_t* __restrict__ fout, int32_t* __restrict__ vsrc,
                                                           long long* counts) {
    const long long i = (long long)blockIdx.x * WELD_THREADS + threadIdx.x;
    if (i < V && used[i]) {
        const uint32_t o = vnum[i];
        vout[3ll * o] = v[3 * i]; vout[3ll * o + 1] = v[3 * i + 1]; vout[3ll * o + 2] = v[3 * i + 2];
        if (vsrc) vsrc[o] = int32_t(i);
    }
    if (i < F && keep[i]) {
        const uint32_t o = fnum[i];
        fout[3ll * o] = int32_t(vnum[f2[3 * i]]);
        fout[3ll * o + 1] = int32_t(vnum[f2[3 * i + 1]]);
        fout[3ll * o + 2] = int32_t(vnum[f2[3 * i + 2]]);
    }
    if (i == 0) {
        counts[0] = V ? (long long)vnum[V - 1] + used[V - 1] : 0;
        counts[1] = F ? (long long)fnum[F - 1] + keep[F - 1] : 0;
    }
}

struct MeshWs {
    uint32_t *table, *rep, *used, *vnum, *f2, *keep, *fnum;
    void* temp;
    size_t temp_bytes, total;
    uint32_t hcap;
};

MeshWs mesh_carve(void* ws, long long V, long long F) {
    MeshWs w{};
    w.hcap = 1024;
    while ((long long)w.hcap < 2 * V + 1024) w.hcap <<= 1;
    size_t tv = 0, tf = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tv, (const uint32_t*)nullptr, (uint32_t*)nullptr, int(std::max(V, 1ll)));
    cub::DeviceScan::ExclusiveSum(nullptr, tf, (const uint32_t*)nullptr, (uint32_t*)nullptr, int(std::max(F, 1ll)));
    w.temp_bytes = std::max(tv, tf);
    uint8_t* b = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    size_t o = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = ws ? b + o : nullptr;
        o = (o + std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        return p;
    };
    w.table = reinterpret_cast<uint32_t*>(take(size_t(w.hcap) * 4));
    w.rep = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.used = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.vnum = reinterpret_cast<uint32_t*>(take(size_t(V) * 4));
    w.f2 = reinterpret_cast<uint32_t*>(take(size_t(F) * 12));
    w.keep = reinterpret_cast<uint32_t*>(take(size_t(F) * 4));
    w.fnum = reinterpret_cast<uint32_t*>(take(size_t(F) * 4));
    w.temp = take(w.temp_bytes);
    w.total = o + 256;
    return w;
}

}  // namespace

extern "C" {

size_t iso_weld_mesh_workspace_size(long long V, long long F) {
    if (V < 0 || F < 0 || V > 0x7fffffffll || F > 0x7fffffffll) return 0;
    return mesh_carve(nullptr, V, F).total;
}

int iso_weld_mesh(const float* vertices, long long V, const int* faces, long long F, float* vout, int* fout,
                  int* vsrc, long long* counts, int* status, void* workspace, size_t workspace_bytes,
                  void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (V < 0 || F < 0 || V > 0x7fffffffll || F > 0x7fffffffll || !counts || !status) return iso::fail_code(ISO_ERR_ARG);
    if ((V && (!vertices || !vout)) || (F && (!faces || !fout))) return iso::fail_code(ISO_ERR_ARG);
    if (workspace_bytes < iso_weld_mesh_workspace_size(V, F)) return iso::fail_code(ISO_ERR_WORKSPACE);
    if (V == 0 || F == 0) return cudaMemsetAsync(counts, 0, 16, st) == cudaSuccess ? ISO_OK : iso::fail_code(ISO_ERR_CUDA);
    const MeshWs w = mesh_carve(workspace, V, F);
    iso::ProfScope ps("weld_mesh", st, 4);
    cudaMemsetAsync(w.table, 0xff, size_t(w.hcap) * 4, st);
    cudaMemsetAsync(w.used, 0, size_t(V) * 4, st);
    weld_insert<<<tiles_for(V), WELD_THREADS, 0, st>>>(vertices, V, w.table, w.hcap - 1, status, nullptr);
    mesh_lookup<<<unsigned((V + WELD_THREADS - 1) / WELD_THREADS), WELD_THREADS, 0, st>>>(vertices, V, w.table,
                                                                                         w.hcap - 1, w.rep);
    mesh_faces<<<unsigned((F + WELD_THREADS - 1) / WELD_THREADS), WELD_THREADS, 0, st>>>(
        reinterpret_cast<const int32_t*>(faces), F, w.rep, w.f2, w.keep, w.used);
    size_t tb = w.temp_bytes;
    if (cub::DeviceScan::ExclusiveSum(w.temp, tb, w.used, w.vnum, int(V), st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    tb = w.temp_bytes;
    if (cub::DeviceScan::ExclusiveSum(w.temp, tb, w.keep, w.fnum, int(F), st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    const long long n = std::max(V, F);
    mesh_write<<<unsigned((n + WELD_THREADS - 1) / WELD_THREADS), WELD_THREADS, 0, st>>>(
        vertices, V, F, w.used, w.vnum, w.keep, w.fnum, w.f2, vout, reinterpret_cast<int32_t*>(fout),
        reinterpret_cast<int32_t*>(vsrc), counts);
    return cudaGetLastError() == cudaSuccess ? ISO_OK : iso::fail_code(ISO_ERR_CUDA);
}

}  // extern "C"
