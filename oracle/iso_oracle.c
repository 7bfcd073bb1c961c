/*
 * iso_oracle.c -- CPU restatement of isoext's marching cubes / dual contouring.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA path is checked
 * against; it is compiled and called only by tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg.  The product never links or calls it.
 *
 * It restates the reference's algorithm step by step in FP32, and welds
 * vertices the way the reference does: by exact position, sorted
 * lexicographically.  Its outputs are therefore the reference's output
 * tensors, bit for bit, in either of two readings of the reference's FP32
 * expressions (ora_set_arith):
 *   1 (default) -- its CUDA build: nvcc's default FMA contraction fuses the
 *                  multiply-adds of the grid position, the lerp, the steps of
 *                  the trilinear interpolant and the dot product (which
 *                  product it fuses is spelt out at each use below; it was
 *                  measured on a restatement of the source compiled by nvcc
 *                  with default flags, tests/nvcc_expr.cu);
 *   0           -- its host build (and its source read literally): every
 *                  operation rounded on its own.
 * The file is built with -ffp-contract=off, so only the explicit fmaf calls
 * fuse.  Reading 0 is pinned against the reference's own code compiled for the
 * host (oracle/_ref, see build_ref.sh) and against the counts published in the
 * reference's notebooks (tests/golden); reading 1 against the nvcc-compiled
 * restatement on the GPU.
 *
 * Reference anchors (paths inside the isoext project):
 *   grid point position         include/utils.cuh:62-80   (get_vtx_pos_op)
 *   cell corners, Morton order  include/utils.cuh:32-60   (idx_to_cell_op)
 *   case number                 include/utils.cuh:82-102  (get_case_num_op)
 *   MC per-cell emission        src/mc/nagae.cu:34-80, src/mc/lorensen.cu:34-80
 *   lerp                        include/math.cuh:77-81
 *   MC driver / NaN removal     src/mc/mc.cu:17-68
 *   vertex welding              src/utils.cu:32-59
 *   intersections               src/its.cu:13-90, 94-159
 *   intersection normals        src/its.cu:170-268
 *   dual quads + neighbours     src/grid/uniform.cu:60-83, include/utils.cuh:104-139
 *   sparse dual quads           src/grid/sparse.cu:181-246
 *   QEF                         src/dc.cu:14-65
 *   least squares via SVD       src/batched_la.cu:152-178 (here: FP64 symmetric
 *                               Jacobi eigen-solve with the same s > tol*s_max rule)
 *   clip / quad split / weld    src/dc.cu:82-157, 162-218
 *
 * Deviation (documented): the reference reads idx_map out of range for quads
 * whose edge lies on a max-side grid face (include/utils.cuh:130 checks lower
 * bounds only).  The oracle treats such neighbours as missing and skips the
 * quad, as the CUDA path does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../isoext_gb300/csrc/luts.h"

typedef struct { float x, y, z; } f3;

static f3 mk(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static f3 add3(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static f3 sub3(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static f3 div3(f3 a, f3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
static f3 divs(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static int eq3(f3 a, f3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
/* the arithmetic reading: 1 = the reference's CUDA build, 0 = its host build */
static int g_fma = 1;
void ora_set_arith(int fma) { g_fma = fma != 0; }
int ora_get_arith(void) { return g_fma; }

/* x * ox + y * oy; the CUDA build fuses the first product, or with swap the
 * second */
static float blend(float x, float ox, float y, float oy, int swap) {
    if (!g_fma) return x * ox + y * oy;
    return swap ? fmaf(y, oy, x * ox) : fmaf(x, ox, y * oy);
}

/* acc + a * b; fused in the CUDA build */
static float acc_mul(float acc, float a, float b) { return g_fma ? fmaf(a, b, acc) : acc + a * b; }

/* dot(a, b) = a.x * b.x + a.y * b.y + a.z * b.z, include/math.cuh;
 * CUDA build: fma(a.z, b.z, fma(a.x, b.x, a.y * b.y)) */
static float dot3(f3 a, f3 b) {
    if (!g_fma) return a.x * b.x + a.y * b.y + a.z * b.z;
    return fmaf(a.z, b.z, fmaf(a.x, b.x, a.y * b.y));
}
static float norm3(f3 a) { return sqrtf(dot3(a, a)); }

/* lerp(t, a, b) = (1 - t) * a + t * b, include/math.cuh:77-81 */
static f3 lerp3(float t, f3 a, f3 b) {
    float u = 1.0f - t;
    return mk(blend(u, a.x, t, b.x, 0), blend(u, a.y, t, b.y, 0), blend(u, a.z, t, b.z, 0));
}

/* one coordinate amin + pos * size; the CUDA build fuses it */
static float pos_coord(float pos, float amin, float size) {
    return g_fma ? fmaf(pos, size, amin) : amin + pos * size;
}

/* Grid point position, include/utils.cuh:62-80. */
static f3 grid_pos(uint32_t ix, uint32_t iy, uint32_t iz, const uint32_t n[3], f3 amin, f3 asize) {
    f3 p = mk((float)ix / (float)(n[0] - 1), (float)iy / (float)(n[1] - 1),
              (float)iz / (float)(n[2] - 1));
    return mk(pos_coord(p.x, amin.x, asize.x), pos_coord(p.y, amin.y, asize.y),
              pos_coord(p.z, amin.z, asize.z));
}

/* The n coordinates of one axis over [amin, amax]. */
void ora_axis_coords(int n, float amin, float amax, float *out) {
    float size = amax - amin;
    for (int i = 0; i < n; i++) out[i] = pos_coord((float)i / (float)(n - 1), amin, size);
}

/* ------------------------------------------------------------------------- */
/* growable arrays                                                            */

typedef struct { void *p; size_t n, cap, esz; } vec_t;

static int vpush(vec_t *v, const void *e) {
    if (v->n == v->cap) {
        size_t nc = v->cap ? v->cap * 2 : 1024;
        void *q = realloc(v->p, nc * v->esz);
        if (!q) return -1;
        v->p = q;
        v->cap = nc;
    }
    memcpy((char *)v->p + v->n * v->esz, e, v->esz);
    v->n++;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* vertex welding, src/utils.cu:32-59                                         */
/* Stable lexicographic sort of the (x, y, z) soup, unique by float equality,  */
/* face index = lower_bound.  The tie-break on the original slot makes qsort   */
/* stable, matching thrust's merge sort.                                      */

typedef struct { f3 p; uint32_t slot; } wsort_t;

static int wcmp(const void *a_, const void *b_) {
    const wsort_t *a = (const wsort_t *)a_, *b = (const wsort_t *)b_;
    if (a->p.x < b->p.x) return -1;
    if (b->p.x < a->p.x) return 1;
    if (a->p.y < b->p.y) return -1;
    if (b->p.y < a->p.y) return 1;
    if (a->p.z < b->p.z) return -1;
    if (b->p.z < a->p.z) return 1;
    return a->slot < b->slot ? -1 : (a->slot > b->slot ? 1 : 0);
}

/* soup: 3*F positions.  Outputs: malloc'd V positions (float[V*3]), faces
 * int32[F*3], and for each vertex the soup slot it was taken from. */
static int weld(const f3 *soup, size_t nslots, float **v_out, int64_t *nv,
                int32_t **f_out, uint32_t **rep_out) {
    wsort_t *w = (wsort_t *)malloc((nslots ? nslots : 1) * sizeof(wsort_t));
    int32_t *f = (int32_t *)malloc((nslots ? nslots : 1) * sizeof(int32_t));
    if (!w || !f) { free(w); free(f); return -1; }
    for (size_t i = 0; i < nslots; i++) { w[i].p = soup[i]; w[i].slot = (uint32_t)i; }
    qsort(w, nslots, sizeof(wsort_t), wcmp);
    size_t nu = 0;
    for (size_t i = 0; i < nslots; i++) {
        if (nu == 0 || !eq3(w[nu - 1].p, w[i].p)) w[nu++] = w[i];
    }
    float *v = (float *)malloc((nu ? nu : 1) * 3 * sizeof(float));
    uint32_t *rep = (uint32_t *)malloc((nu ? nu : 1) * sizeof(uint32_t));
    if (!v || !rep) { free(w); free(f); free(v); free(rep); return -1; }
    for (size_t i = 0; i < nu; i++) {
        v[3 * i] = w[i].p.x; v[3 * i + 1] = w[i].p.y; v[3 * i + 2] = w[i].p.z;
        rep[i] = w[i].slot;
    }
    for (size_t s = 0; s < nslots; s++) {
        /* lower_bound with the lexicographic less-than on positions */
        size_t lo = 0, hi = nu;
        f3 q = soup[s];
        while (lo < hi) {
            size_t mid = (lo + hi) / 2;
            f3 m = w[mid].p;
            int less = m.x < q.x || (!(q.x < m.x) && (m.y < q.y || (!(q.y < m.y) && m.z < q.z)));
            if (less) lo = mid + 1; else hi = mid;
        }
        f[s] = (int32_t)lo;
    }
    free(w);
    *v_out = v;
    *nv = (int64_t)nu;
    *f_out = f;
    *rep_out = rep;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* marching cubes                                                             */

typedef struct {
    float val[8];
    f3 pos[8];
    uint32_t pid[8]; /* global point id of each corner (for vertex provenance) */
} cell_t;

typedef struct {
    vec_t soup;  /* f3 per slot */
    vec_t edge;  /* uint32 pair (p0, p1) per slot */
} mc_acc_t;

/* Process one cell: src/mc/nagae.cu:34-80. */
static int mc_cell(const cell_t *c, float level, int method, mc_acc_t *acc) {
    unsigned cs = 0;
    for (int i = 0; i < 8; i++) cs |= (unsigned)(c->val[i] - level < 0) << i;
    if (cs == 0 || cs == 255) return 0;
    int st = ISO_EDGE_STATUS[cs];
    f3 cube_v[12];
    for (int e = 0; e < 12; e++) {
        if (st & (1 << e)) {
            int a = ISO_EDGE_CORNERS[2 * e], b = ISO_EDGE_CORNERS[2 * e + 1];
            float denom = c->val[b] - c->val[a];
            float t = (denom != 0.0f) ? (level - c->val[a]) / denom : 0.0f;
            cube_v[e] = lerp3(t, c->pos[a], c->pos[b]);
        }
    }
    const signed char *tri = method ? ISO_TRI_LORENSEN : ISO_TRI_NAGAE;
    int ml = method ? 3 * ISO_LORENSEN_MAX_TRI : 3 * ISO_NAGAE_MAX_TRI;
    for (int s = 0; s < ml; s += 3) {
        const signed char *t = tri + cs * ml + s;
        if (t[0] == -1) break;
        f3 v0 = cube_v[(int)t[0]], v1 = cube_v[(int)t[1]], v2 = cube_v[(int)t[2]];
        if (!eq3(v0, v1) && !eq3(v0, v2) && !eq3(v1, v2)) {
            for (int k = 0; k < 3; k++) {
                int e = t[k];
                uint32_t pe[2] = {c->pid[ISO_EDGE_CORNERS[2 * e]], c->pid[ISO_EDGE_CORNERS[2 * e + 1]]};
                if (vpush(&acc->soup, &cube_v[e]) || vpush(&acc->edge, pe)) return -1;
            }
        }
    }
    return 0;
}

static int mc_finish(mc_acc_t *acc, float **v, int64_t *nv, int32_t **f, int64_t *nf,
                     uint32_t **vedge) {
    uint32_t *rep = NULL;
    f3 *soup = (f3 *)acc->soup.p;
    if (weld(soup, acc->soup.n, v, nv, f, &rep)) return -1;
    *nf = (int64_t)(acc->soup.n / 3);
    if (vedge) {
        uint32_t *ve = (uint32_t *)malloc((*nv ? *nv : 1) * 2 * sizeof(uint32_t));
        if (!ve) return -1;
        for (int64_t i = 0; i < *nv; i++) {
            memcpy(ve + 2 * i, (uint32_t *)acc->edge.p + 2 * (size_t)rep[i], 2 * sizeof(uint32_t));
        }
        *vedge = ve;
    }
    free(rep);
    free(acc->soup.p);
    free(acc->edge.p);
    return 0;
}

static void dense_cell(const float *vals, const uint32_t n[3], f3 amin, f3 asize,
                       uint32_t x, uint32_t y, uint32_t z, cell_t *c) {
    for (int k = 0; k < 8; k++) {
        uint32_t ix = x + (k >> 2), iy = y + ((k >> 1) & 1), iz = z + (k & 1);
        uint32_t pid = (ix * n[1] + iy) * n[2] + iz;
        c->pid[k] = pid;
        c->val[k] = vals[pid];
        c->pos[k] = grid_pos(ix, iy, iz, n, amin, asize);
    }
}

/* Dense marching cubes, src/mc/mc.cu:17-68.  vedge (optional) receives, per
 * output vertex, the point ids (p0, p1) of the grid edge it came from. */
int ora_mc_dense(const float *vals, int nx, int ny, int nz, const float *aabb_min,
                 const float *aabb_max, float level, int method, float **v, int64_t *nv,
                 int32_t **f, int64_t *nf, uint32_t **vedge) {
    uint32_t n[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
    f3 amin = mk(aabb_min[0], aabb_min[1], aabb_min[2]);
    f3 asize = sub3(mk(aabb_max[0], aabb_max[1], aabb_max[2]), amin);
    mc_acc_t acc = {{NULL, 0, 0, sizeof(f3)}, {NULL, 0, 0, 2 * sizeof(uint32_t)}};
    cell_t c;
    for (uint32_t x = 0; x + 1 < n[0]; x++)
        for (uint32_t y = 0; y + 1 < n[1]; y++)
            for (uint32_t z = 0; z + 1 < n[2]; z++) {
                /* cheap reject before building positions */
                size_t b = ((size_t)x * n[1] + y) * n[2] + z;
                size_t o[8] = {0, 1, n[2], n[2] + 1, (size_t)n[1] * n[2], (size_t)n[1] * n[2] + 1,
                               (size_t)n[1] * n[2] + n[2], (size_t)n[1] * n[2] + n[2] + 1};
                unsigned cs = 0;
                for (int k = 0; k < 8; k++) cs |= (unsigned)(vals[b + o[k]] - level < 0) << k;
                if (cs == 0 || cs == 255) continue;
                dense_cell(vals, n, amin, asize, x, y, z, &c);
                if (mc_cell(&c, level, method, &acc)) return -1;
            }
    return mc_finish(&acc, v, nv, f, nf, vedge);
}

/* Sparse cells: cell c has linear index cell_ids[c] over the (n-1)^3 cell
 * lattice and its own 8 corner values values[8c..8c+7] (Morton order).
 * Positions come from the global point ids (src/grid/sparse.cu:21-36). */
static void sparse_cell(const int32_t *ids, const float *values, int64_t c, const uint32_t n[3],
                        f3 amin, f3 asize, cell_t *out) {
    uint32_t i = (uint32_t)ids[c];
    uint32_t z = i % (n[2] - 1);
    i /= (n[2] - 1);
    uint32_t y = i % (n[1] - 1);
    uint32_t x = i / (n[1] - 1);
    for (int k = 0; k < 8; k++) {
        uint32_t ix = x + (k >> 2), iy = y + ((k >> 1) & 1), iz = z + (k & 1);
        out->pid[k] = (ix * n[1] + iy) * n[2] + iz;
        out->val[k] = values[8 * c + k];
        out->pos[k] = grid_pos(ix, iy, iz, n, amin, asize);
    }
}

/* Sparse marching cubes: the MC driver over SparseGrid (cells = iota,
 * src/grid/sparse.cu:61-69).  cell_ids must be sorted and unique, as
 * SparseGrid keeps them. */
int ora_mc_sparse(const int32_t *cell_ids, const float *values, int64_t ncells, int nx, int ny,
                  int nz, const float *aabb_min, const float *aabb_max, float level, int method,
                  float **v, int64_t *nv, int32_t **f, int64_t *nf, uint32_t **vedge) {
    uint32_t n[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
    f3 amin = mk(aabb_min[0], aabb_min[1], aabb_min[2]);
    f3 asize = sub3(mk(aabb_max[0], aabb_max[1], aabb_max[2]), amin);
    mc_acc_t acc = {{NULL, 0, 0, sizeof(f3)}, {NULL, 0, 0, 2 * sizeof(uint32_t)}};
    cell_t c;
    for (int64_t i = 0; i < ncells; i++) {
        sparse_cell(cell_ids, values, i, n, amin, asize, &c);
        if (mc_cell(&c, level, method, &acc)) return -1;
    }
    return mc_finish(&acc, v, nv, f, nf, vedge);
}

/* ------------------------------------------------------------------------- */
/* intersections and normals                                                  */

typedef struct {
    int64_t ncross, nactive;
    float *points;     /* [K,3] */
    float *normals;    /* [K,3] */
    uint32_t *edges;   /* [K,2] point ids (p0 < p1) */
    uint8_t *is_out;   /* [K]   v0 <= v1 */
    uint32_t *cells;   /* [A]   active cell linear ids (dense lattice) */
    uint32_t *offsets; /* [A+1] CSR */
} ora_its_t;

/* trilinear interpolation, src/its.cu:170-184.  swap_low_z: in the CUDA build
 * the two x = 0 steps along z fuse their second product; nvcc does that for the
 * four stencil samples at the crossing's own z, which share those steps. */
static float trilin(f3 t, const float *cv, int swap_low_z) {
    float oz = 1 - t.z, oy = 1 - t.y, ox = 1 - t.x;
    float c00 = blend(cv[0], oz, cv[1], t.z, swap_low_z);
    float c01 = blend(cv[2], oz, cv[3], t.z, swap_low_z);
    float c10 = blend(cv[4], oz, cv[5], t.z, 0);
    float c11 = blend(cv[6], oz, cv[7], t.z, 0);
    float c0 = blend(c00, oy, c01, t.y, 0);
    float c1 = blend(c10, oy, c11, t.y, 0);
    return blend(c0, ox, c1, t.x, 0);
}

/* normal at one crossing from the cell's corners, src/its.cu:186-268 */
static f3 cell_normal(const cell_t *c, f3 p) {
    f3 cmin = c->pos[0];
    f3 csz = sub3(c->pos[7], c->pos[0]);
    f3 t = div3(sub3(p, cmin), csz);
    t.x = fmaxf(0.01f, fminf(0.99f, t.x));
    t.y = fmaxf(0.01f, fminf(0.99f, t.y));
    t.z = fmaxf(0.01f, fminf(0.99f, t.z));
    float eps = 0.02f;
    f3 tpx = mk(fminf(t.x + eps, 0.99f), t.y, t.z), tmx = mk(fmaxf(t.x - eps, 0.01f), t.y, t.z);
    f3 tpy = mk(t.x, fminf(t.y + eps, 0.99f), t.z), tmy = mk(t.x, fmaxf(t.y - eps, 0.01f), t.z);
    f3 tpz = mk(t.x, t.y, fminf(t.z + eps, 0.99f)), tmz = mk(t.x, t.y, fmaxf(t.z - eps, 0.01f));
    float dx = (trilin(tpx, c->val, 1) - trilin(tmx, c->val, 1)) / ((tpx.x - tmx.x) * csz.x);
    float dy = (trilin(tpy, c->val, 1) - trilin(tmy, c->val, 1)) / ((tpy.y - tmy.y) * csz.y);
    float dz = (trilin(tpz, c->val, 0) - trilin(tmz, c->val, 0)) / ((tpz.z - tmz.z) * csz.z);
    f3 g = mk(dx, dy, dz);
    float len = norm3(g);
    return len > 1e-8f ? divs(g, len) : mk(0.0f, 0.0f, 1.0f);
}

static int its_cell(const cell_t *c, float level, int with_normals, vec_t *pts, vec_t *nrm,
                    vec_t *edg, vec_t *out) {
    unsigned cs = 0;
    for (int i = 0; i < 8; i++) cs |= (unsigned)(c->val[i] - level < 0) << i;
    int st = ISO_EDGE_STATUS[cs];
    int cnt = 0;
    for (int e = 0; e < 12; e++) {
        if (!(st & (1 << e))) continue;
        int a = ISO_EDGE_CORNERS[2 * e], b = ISO_EDGE_CORNERS[2 * e + 1];
        uint32_t pe[2] = {c->pid[a], c->pid[b]};
        uint8_t io = c->val[a] <= c->val[b];
        float denom = c->val[b] - c->val[a];
        float t = (denom != 0.0f) ? (level - c->val[a]) / denom : 0.0f;
        f3 p = lerp3(t, c->pos[a], c->pos[b]);
        f3 nn = with_normals ? cell_normal(c, p) : mk(0, 0, 0);
        if (vpush(pts, &p) || vpush(nrm, &nn) || vpush(edg, pe) || vpush(out, &io)) return -1;
        cnt++;
    }
    return cnt;
}

/* get_intersection over a dense grid, src/its.cu:94-159 (+ normals). */
int ora_intersection_dense(const float *vals, int nx, int ny, int nz, const float *aabb_min,
                           const float *aabb_max, float level, int with_normals, ora_its_t *its) {
    uint32_t n[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
    f3 amin = mk(aabb_min[0], aabb_min[1], aabb_min[2]);
    f3 asize = sub3(mk(aabb_max[0], aabb_max[1], aabb_max[2]), amin);
    vec_t pts = {NULL, 0, 0, sizeof(f3)}, nrm = {NULL, 0, 0, sizeof(f3)};
    vec_t edg = {NULL, 0, 0, 2 * sizeof(uint32_t)}, io = {NULL, 0, 0, 1};
    vec_t cel = {NULL, 0, 0, sizeof(uint32_t)}, off = {NULL, 0, 0, sizeof(uint32_t)};
    uint32_t zero = 0;
    if (vpush(&off, &zero)) return -1;
    cell_t c;
    uint32_t cid = 0;
    for (uint32_t x = 0; x + 1 < n[0]; x++)
        for (uint32_t y = 0; y + 1 < n[1]; y++)
            for (uint32_t z = 0; z + 1 < n[2]; z++, cid++) {
                size_t b = ((size_t)x * n[1] + y) * n[2] + z;
                size_t o[8] = {0, 1, n[2], n[2] + 1, (size_t)n[1] * n[2], (size_t)n[1] * n[2] + 1,
                               (size_t)n[1] * n[2] + n[2], (size_t)n[1] * n[2] + n[2] + 1};
                unsigned cs = 0;
                for (int k = 0; k < 8; k++) cs |= (unsigned)(vals[b + o[k]] - level < 0) << k;
                if (ISO_EDGE_STATUS[cs] == 0) continue;
                dense_cell(vals, n, amin, asize, x, y, z, &c);
                if (its_cell(&c, level, with_normals, &pts, &nrm, &edg, &io) < 0) return -1;
                uint32_t end = (uint32_t)pts.n;
                if (vpush(&cel, &cid) || vpush(&off, &end)) return -1;
            }
    its->ncross = (int64_t)pts.n;
    its->nactive = (int64_t)cel.n;
    its->points = (float *)pts.p;
    its->normals = (float *)nrm.p;
    its->edges = (uint32_t *)edg.p;
    its->is_out = (uint8_t *)io.p;
    its->cells = (uint32_t *)cel.p;
    its->offsets = (uint32_t *)off.p;
    return 0;
}

/* get_intersection over a sparse grid: active entries are positions in the
 * sparse cell list; edges are stored as sparse point ids 8c+k like the
 * reference's (cells = iota) and converted by the DC routine. */
int ora_intersection_sparse(const int32_t *cell_ids, const float *values, int64_t ncells, int nx,
                            int ny, int nz, const float *aabb_min, const float *aabb_max,
                            float level, int with_normals, ora_its_t *its) {
    uint32_t n[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
    f3 amin = mk(aabb_min[0], aabb_min[1], aabb_min[2]);
    f3 asize = sub3(mk(aabb_max[0], aabb_max[1], aabb_max[2]), amin);
    vec_t pts = {NULL, 0, 0, sizeof(f3)}, nrm = {NULL, 0, 0, sizeof(f3)};
    vec_t edg = {NULL, 0, 0, 2 * sizeof(uint32_t)}, io = {NULL, 0, 0, 1};
    vec_t cel = {NULL, 0, 0, sizeof(uint32_t)}, off = {NULL, 0, 0, sizeof(uint32_t)};
    uint32_t zero = 0;
    if (vpush(&off, &zero)) return -1;
    cell_t c;
    for (int64_t i = 0; i < ncells; i++) {
        sparse_cell(cell_ids, values, i, n, amin, asize, &c);
        unsigned cs = 0;
        for (int k = 0; k < 8; k++) cs |= (unsigned)(c.val[k] - level < 0) << k;
        if (ISO_EDGE_STATUS[cs] == 0) continue;
        for (int k = 0; k < 8; k++) c.pid[k] = (uint32_t)(8 * i + k);
        if (its_cell(&c, level, with_normals, &pts, &nrm, &edg, &io) < 0) return -1;
        uint32_t end = (uint32_t)pts.n, ci = (uint32_t)i;
        if (vpush(&cel, &ci) || vpush(&off, &end)) return -1;
    }
    its->ncross = (int64_t)pts.n;
    its->nactive = (int64_t)cel.n;
    its->points = (float *)pts.p;
    its->normals = (float *)nrm.p;
    its->edges = (uint32_t *)edg.p;
    its->is_out = (uint8_t *)io.p;
    its->cells = (uint32_t *)cel.p;
    its->offsets = (uint32_t *)off.p;
    return 0;
}

void ora_its_free(ora_its_t *its) {
    free(its->points); free(its->normals); free(its->edges);
    free(its->is_out); free(its->cells); free(its->offsets);
    memset(its, 0, sizeof(*its));
}

/* ------------------------------------------------------------------------- */
/* dual contouring                                                            */

/* Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (Golub & Van
 * Loan, Matrix Computations, sec. 8.5), FP64.  a is overwritten. */
static void jacobi3(double a[3][3], double w[3], double q[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) q[i][j] = (i == j);
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double tot = off + a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int r = p + 1; r < 3; r++) {
                if (a[p][r] == 0.0) continue;
                double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    double akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 3; k++) {
                    double qkp = q[k][p], qkr = q[k][r];
                    q[k][p] = c * qkp - s * qkr;
                    q[k][r] = s * qkp + c * qkr;
                }
            }
    }
    for (int i = 0; i < 3; i++) w[i] = a[i][i];
}

/* x = pinv(A) b with singular values s_i <= tol * s_max dropped
 * (src/batched_la.cu:152-178).  For symmetric A the singular values are |w_i|. */
static void lsq_sym(const float ata[9], const float atb[3], float tol, double x[3]) {
    double a[3][3], w[3], q[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[i][j] = ata[3 * i + j];
    jacobi3(a, w, q);
    double smax = 0;
    for (int i = 0; i < 3; i++) smax = fmax(smax, fabs(w[i]));
    x[0] = x[1] = x[2] = 0;
    for (int i = 0; i < 3; i++) {
        /* the reference compares float s_i with float (tol * s_max) */
        float si = (float)fabs(w[i]);
        float thr = tol * (float)smax;
        if (!(si > thr)) continue;
        double qb = q[0][i] * atb[0] + q[1][i] * atb[1] + q[2][i] * atb[2];
        double coef = qb / w[i];
        for (int k = 0; k < 3; k++) x[k] += coef * q[k][i];
    }
}

typedef struct { uint32_t p0, p1; uint8_t io; uint32_t ord; } qedge_t;

static int qcmp(const void *a_, const void *b_) {
    const qedge_t *a = (const qedge_t *)a_, *b = (const qedge_t *)b_;
    if (a->p0 != b->p0) return a->p0 < b->p0 ? -1 : 1;
    if (a->p1 != b->p1) return a->p1 < b->p1 ? -1 : 1;
    return a->ord < b->ord ? -1 : (a->ord > b->ord ? 1 : 0);
}

/* The QEF of one cell's crossings [b0, b1) (src/dc.cu:26-62): ata and atb
 * (zeroed by the caller) in the current arithmetic reading. */
static void qef_cell(const float *points, const float *normals, uint32_t b0, uint32_t b1, float reg,
                     float *ata, float *atb) {
    f3 pavg = mk(0, 0, 0);
    for (uint32_t i = b0; i < b1; i++) {
        f3 nn = mk(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
        f3 p = mk(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
        float d = dot3(nn, p);
        pavg = add3(pavg, p);
        /* acc += a * b; the CUDA build fuses each into fma(a, b, acc) */
        ata[0] = acc_mul(ata[0], nn.x, nn.x); ata[1] = acc_mul(ata[1], nn.x, nn.y);
        ata[2] = acc_mul(ata[2], nn.x, nn.z); ata[3] = acc_mul(ata[3], nn.y, nn.x);
        ata[4] = acc_mul(ata[4], nn.y, nn.y); ata[5] = acc_mul(ata[5], nn.y, nn.z);
        ata[6] = acc_mul(ata[6], nn.z, nn.x); ata[7] = acc_mul(ata[7], nn.z, nn.y);
        ata[8] = acc_mul(ata[8], nn.z, nn.z);
        atb[0] = acc_mul(atb[0], nn.x, d); /* += (n * dot(n, p)).x */
        atb[1] = acc_mul(atb[1], nn.y, d);
        atb[2] = acc_mul(atb[2], nn.z, d);
    }
    pavg = divs(pavg, (float)(b1 - b0));
    ata[0] += reg; ata[4] += reg; ata[8] += reg;
    atb[0] = acc_mul(atb[0], reg, pavg.x);
    atb[1] = acc_mul(atb[1], reg, pavg.y);
    atb[2] = acc_mul(atb[2], reg, pavg.z);
}

/* The QEFs of A cells with CSR offsets: ata [A, 9], atb [A, 3]. */
void ora_qef(const float *points, const float *normals, const uint32_t *offsets, int64_t A, float reg,
             float *ata, float *atb) {
    for (int64_t a = 0; a < A; a++) {
        memset(ata + 9 * a, 0, 9 * sizeof(float));
        memset(atb + 3 * a, 0, 3 * sizeof(float));
        qef_cell(points, normals, offsets[a], offsets[a + 1], reg, ata + 9 * a, atb + 3 * a);
    }
}

/* Dual contouring (src/dc.cu:162-218) over a dense grid (sparse == 0) or a
 * sparse grid (sparse == 1: cell_ids/values describe the sparse cells and the
 * intersection's edges and cells are sparse-local).  dual_out (optional)
 * receives the FP64 QEF solution of every active cell before clipping. */
int ora_dc(const float *vals, const int32_t *cell_ids, int64_t nsparse, int sparse, int nx,
           int ny, int nz, const float *aabb_min, const float *aabb_max, const ora_its_t *its,
           float reg, float svd_tol, float **v, int64_t *nv, int32_t **f, int64_t *nf,
           double **dual_out) {
    uint32_t n[3] = {(uint32_t)nx, (uint32_t)ny, (uint32_t)nz};
    f3 amin = mk(aabb_min[0], aabb_min[1], aabb_min[2]);
    f3 asize = sub3(mk(aabb_max[0], aabb_max[1], aabb_max[2]), amin);
    int64_t A = its->nactive, K = its->ncross;
    uint32_t ncell = (n[0] - 1) * (n[1] - 1) * (n[2] - 1);

    /* --- dual quads: dedupe edges by (p0, p1), keep first is_out --- */
    qedge_t *qe = (qedge_t *)malloc((K ? K : 1) * sizeof(qedge_t));
    if (!qe) return -1;
    for (int64_t i = 0; i < K; i++) {
        uint32_t p0 = its->edges[2 * i], p1 = its->edges[2 * i + 1];
        if (sparse) { /* sparse point id -> dense lattice point id */
            uint32_t c = p0 / 8, k0 = p0 % 8, k1 = p1 % 8, cc = (uint32_t)cell_ids[c];
            uint32_t z = cc % (n[2] - 1), t = cc / (n[2] - 1);
            uint32_t y = t % (n[1] - 1), x = t / (n[1] - 1);
            p0 = ((x + (k0 >> 2)) * n[1] + y + ((k0 >> 1) & 1)) * n[2] + z + (k0 & 1);
            p1 = ((x + (k1 >> 2)) * n[1] + y + ((k1 >> 1) & 1)) * n[2] + z + (k1 & 1);
        }
        qe[i].p0 = p0; qe[i].p1 = p1; qe[i].io = its->is_out[i]; qe[i].ord = (uint32_t)i;
    }
    qsort(qe, (size_t)K, sizeof(qedge_t), qcmp);
    int64_t E = 0;
    for (int64_t i = 0; i < K; i++)
        if (E == 0 || qe[E - 1].p0 != qe[i].p0 || qe[E - 1].p1 != qe[i].p1) qe[E++] = qe[i];

    /* --- QEF per active cell, src/dc.cu:14-65 --- */
    float *dual = (float *)malloc((A ? A : 1) * 3 * sizeof(float));
    double *d64 = (double *)malloc((A ? A : 1) * 3 * sizeof(double));
    if (!dual || !d64) { free(qe); free(dual); free(d64); return -1; }
    for (int64_t a = 0; a < A; a++) {
        float ata[9] = {0}, atb[3] = {0};
        qef_cell(its->points, its->normals, its->offsets[a], its->offsets[a + 1], reg, ata, atb);
        double x[3];
        lsq_sym(ata, atb, svd_tol, x);
        d64[3 * a] = x[0]; d64[3 * a + 1] = x[1]; d64[3 * a + 2] = x[2];
        /* clip to the cell box, src/dc.cu:82-99 */
        cell_t c;
        if (sparse) {
            sparse_cell(cell_ids, vals, (int64_t)its->cells[a], n, amin, asize, &c);
        } else {
            uint32_t cc = its->cells[a];
            uint32_t z = cc % (n[2] - 1), t = cc / (n[2] - 1);
            dense_cell(vals, n, amin, asize, t / (n[1] - 1), t % (n[1] - 1), z, &c);
        }
        f3 lo = c.pos[0], hi = c.pos[7];
        f3 xf = mk((float)x[0], (float)x[1], (float)x[2]);
        dual[3 * a] = fminf(fmaxf(xf.x, lo.x), hi.x);
        dual[3 * a + 1] = fminf(fmaxf(xf.y, lo.y), hi.y);
        dual[3 * a + 2] = fminf(fmaxf(xf.z, lo.z), hi.z);
    }

    /* --- cell -> dual vertex map --- */
    /* dense: lattice cell id -> active index; sparse: lattice cell id ->
     * sparse index -> active index (two maps in the reference). */
    int32_t *amap = (int32_t *)malloc((size_t)(ncell ? ncell : 1) * sizeof(int32_t));
    if (!amap) { free(qe); free(dual); free(d64); return -1; }
    for (uint32_t i = 0; i < ncell; i++) amap[i] = -1;
    for (int64_t a = 0; a < A; a++) {
        uint32_t lat = sparse ? (uint32_t)cell_ids[its->cells[a]] : its->cells[a];
        if (lat < ncell) amap[lat] = (int32_t)a; /* ids past the lattice have no quads */
    }

    /* --- quads -> triangle soup, src/dc.cu:101-157 --- */
    f3 *soup = (f3 *)malloc((E ? E : 1) * 6 * sizeof(f3));
    if (!soup) { free(qe); free(dual); free(d64); free(amap); return -1; }
    size_t ns = 0;
    for (int64_t e = 0; e < E; e++) {
        uint32_t p0 = qe[e].p0, p1 = qe[e].p1;
        uint32_t z = p0 % n[2], t = p0 / n[2];
        uint32_t y = t % n[1], x = t / n[1];
        uint32_t d = p1 - p0;
        /* edge_neighbors_table, src/shared_luts.cu:78-81 */
        static const int nbx[3][4][3] = {
            {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}},
            {{0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 0, 0}},
            {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}},
        };
        int ax = (d == n[1] * n[2]) ? 0 : (d == n[2] ? 1 : 2);
        int32_t q[4];
        int skip = 0;
        for (int i = 0; i < 4; i++) {
            int cx = (int)x - nbx[ax][i][0], cy = (int)y - nbx[ax][i][1], cz = (int)z - nbx[ax][i][2];
            if (cx < 0 || cy < 0 || cz < 0 || cx >= (int)n[0] - 1 || cy >= (int)n[1] - 1 ||
                cz >= (int)n[2] - 1) { skip = 1; break; }
            uint32_t lat = ((uint32_t)cx * (n[1] - 1) + (uint32_t)cy) * (n[2] - 1) + (uint32_t)cz;
            q[i] = amap[lat];
            if (q[i] < 0) { skip = 1; break; }
        }
        if (skip) continue;
        if (!qe[e].io) { int32_t s0 = q[0], s1 = q[1]; q[0] = q[3]; q[1] = q[2]; q[2] = s1; q[3] = s0; }
        f3 v0 = mk(dual[3 * q[0]], dual[3 * q[0] + 1], dual[3 * q[0] + 2]);
        f3 v1 = mk(dual[3 * q[1]], dual[3 * q[1] + 1], dual[3 * q[1] + 2]);
        f3 v2 = mk(dual[3 * q[2]], dual[3 * q[2] + 1], dual[3 * q[2] + 2]);
        f3 v3 = mk(dual[3 * q[3]], dual[3 * q[3] + 1], dual[3 * q[3] + 2]);
        if (norm3(sub3(v0, v2)) > norm3(sub3(v1, v3))) {
            soup[ns++] = v1; soup[ns++] = v3; soup[ns++] = v0;
            soup[ns++] = v3; soup[ns++] = v1; soup[ns++] = v2;
        } else {
            soup[ns++] = v2; soup[ns++] = v0; soup[ns++] = v1;
            soup[ns++] = v0; soup[ns++] = v2; soup[ns++] = v3;
        }
    }
    uint32_t *rep = NULL;
    int rc = weld(soup, ns, v, nv, f, &rep);
    *nf = (int64_t)(ns / 3);
    free(rep);
    free(soup); free(qe); free(dual); free(amap);
    if (dual_out) *dual_out = d64; else free(d64);
    return rc;
}

void ora_free(void *p) { free(p); }
