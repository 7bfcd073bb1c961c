// Dual-contouring arithmetic shared by the forward kernels (dc_dense.cu) and
// the backward kernels (backward.cu): grid positions, cell corners, the
// trilinear interpolant and its normal stencil, the 3x3 symmetric eigen-solve.
// Every operation is rounded as in the reference's code (src/its.cu:170-268,
// src/dc.cu:14-99), so a kernel that recomputes a forward quantity gets the
// same bits.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace {

struct Grid3 {
    int nx, ny, nz;
    float amin[3], asize[3];
    bool fma;  // arithmetic reading (iso::arith_fma at the call)
};

__device__ __forceinline__ float coord(const Grid3& g, int axis, uint32_t i) {
    const uint32_t n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
    return iso::grid_coord(i, n, g.amin[axis], g.asize[axis], g.fma);
}

struct CellCorners {
    float v[8];
    float p[8][3];
    bool fma;  // the grid's arithmetic reading
};

__device__ __forceinline__ void load_cell(const float* vals, const Grid3& g, int cx, int cy, int cz,
                                          CellCorners& cc) {
    cc.fma = g.fma;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int x = cx + (k >> 2), y = cy + ((k >> 1) & 1), z = cz + (k & 1);
        cc.v[k] = __ldg(vals + ((long long)x * g.ny + y) * g.nz + z);
        cc.p[k][0] = coord(g, 0, uint32_t(x));
        cc.p[k][1] = coord(g, 1, uint32_t(y));
        cc.p[k][2] = coord(g, 2, uint32_t(z));
    }
}

// load_cell with the corner positions from a table of the grid's coordinates
// (x, then y, then z; the same bits as coord()).
__device__ __forceinline__ void load_cell_table(const float* vals, const Grid3& g, const float* __restrict__ gc,
                                                int cx, int cy, int cz, CellCorners& cc) {
    cc.fma = g.fma;
    const float x0 = gc[cx], x1 = gc[cx + 1];
    const float y0 = gc[g.nx + cy], y1 = gc[g.nx + cy + 1];
    const float z0 = gc[g.nx + g.ny + cz], z1 = gc[g.nx + g.ny + cz + 1];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int x = cx + (k >> 2), y = cy + ((k >> 1) & 1), z = cz + (k & 1);
        cc.v[k] = __ldg(vals + ((long long)x * g.ny + y) * g.nz + z);
        cc.p[k][0] = (k >> 2) ? x1 : x0;
        cc.p[k][1] = ((k >> 1) & 1) ? y1 : y0;
        cc.p[k][2] = (k & 1) ? z1 : z0;
    }
}

// Normal at crossing point p of a cell (src/its.cu:186-268).
__device__ __forceinline__ void cell_normal(const CellCorners& cc, const float* p, float* n) {
    iso::stencil_normal(cc.v, cc.p[0], cc.p[7], p, n, cc.fma);
}

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (Golub & Van
// Loan, sec. 8.5), FP32.  Each rotation annihilates its pair exactly (a_pr = 0,
// a_pp -= t a_pr, a_rr += t a_pr, the third row and column rotated), so the
// off-diagonal mass falls quadratically to zero instead of stalling at FP32
// rounding.  a is destroyed; w = eigenvalues, q = eigenvectors (columns).
__device__ __forceinline__ void jacobi3f(float a[3][3], float w[3], float q[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) q[i][j] = i == j ? 1.0f : 0.0f;
    for (int sweep = 0; sweep < 12; ++sweep) {
        const float off = fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]);
        const float diag = fabsf(a[0][0]) + fabsf(a[1][1]) + fabsf(a[2][2]);
        if (off <= 1e-9f * diag || off == 0.0f) break;
#pragma unroll
        for (int pr = 0; pr < 3; ++pr) {
            const int p = pr == 2 ? 1 : 0, r = pr == 0 ? 1 : 2, k = 3 - p - r;
            const float apr = a[p][r];
            if (apr == 0.0f) continue;
            const float theta = (a[r][r] - a[p][p]) / (2.0f * apr);
            const float t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
            const float c = rsqrtf(t * t + 1.0f), s = t * c;
            const float tapr = t * apr;
            a[p][p] -= tapr;
            a[r][r] += tapr;
            a[p][r] = a[r][p] = 0.0f;
            const float akp = a[k][p], akr = a[k][r];
            a[k][p] = a[p][k] = c * akp - s * akr;
            a[k][r] = a[r][k] = s * akp + c * akr;
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const float qmp = q[m][p], qmr = q[m][r];
                q[m][p] = c * qmp - s * qmr;
                q[m][r] = s * qmp + c * qmr;
            }
        }
    }
    w[0] = a[0][0]; w[1] = a[1][1]; w[2] = a[2][2];
}

// x += pinv(A) r with the eigen-decomposition (w, q) and the kept mask.
__device__ __forceinline__ void apply_pinv_f(const float w[3], const float q[3][3], unsigned keep, const float r[3],
                                             float x[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (!((keep >> i) & 1u)) continue;
        const float c = (q[0][i] * r[0] + q[1][i] * r[1] + q[2][i] * r[2]) / w[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) x[k] += c * q[k][i];
    }
}

// b - row . x with FP32 error-free transformations (Dekker's product by fma,
// Knuth's two-sum), rounded once at the end: the residual to about twice FP32's
// precision, which is what the refinement step needs (GB300's FP64 rate is a
// small fraction of its FP32 rate).
__device__ __forceinline__ float residual_ff(float b, const float* row, const float* x) {
    float s = b, e = 0.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const float p = __fmul_rn(row[j], x[j]);
        const float pe = fmaf(row[j], x[j], -p);  // row[j] * x[j] = p + pe exactly
        const float t = __fsub_rn(s, p);           // two-sum of s and -p
        const float bb = __fsub_rn(t, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(-p, bb));
        s = t;
        e = __fadd_rn(e, __fsub_rn(err, pe));
    }
    return __fadd_rn(s, e);
}

// QEF of a cell: normal equations of the crossings' planes plus reg times the
// distance to their mean point, accumulated as src/dc.cu:26-62 does (crossings
// in order, in the grid's arithmetic reading: the CUDA build fuses the dot
// product as the norm, and each `+= a * b` into fma(a, b, acc)); solved by the
// pseudo-inverse of the 3x3 system with the threshold svd_tol * largest
// singular value (src/batched_la.cu:152-178), from an FP32 eigen-decomposition
// refined once with a double-FP32 residual.
struct Qef {
    float ata[9], atb[3];  // the system (reg included after qef_finish)
    float px, py, pz;      // sum of the points
    float w[3], q[3][3];   // its eigenvalues and eigenvectors (columns)
    unsigned keep;         // eigenvalues above the threshold
    double x[3];           // the solution before clipping
    bool fma;              // arithmetic reading of the accumulation
};

__device__ __forceinline__ void qef_init(Qef& Q, bool fma) {
#pragma unroll
    for (int i = 0; i < 9; ++i) Q.ata[i] = 0.0f;
    Q.atb[0] = Q.atb[1] = Q.atb[2] = 0.0f;
    Q.px = Q.py = Q.pz = 0.0f;
    Q.fma = fma;
}

// acc += a * b
__device__ __forceinline__ float acc_mul(float acc, float a, float b, bool fma) {
    return fma ? __fmaf_rn(a, b, acc) : __fadd_rn(acc, __fmul_rn(a, b));
}

// One crossing: point (qx, qy, qz), normal (nx, ny, nz).
__device__ __forceinline__ void qef_add(Qef& Q, float qx, float qy, float qz, float nx, float ny, float nz) {
    const float d = Q.fma ? __fmaf_rn(nz, qz, __fmaf_rn(nx, qx, __fmul_rn(ny, qy)))
                          : __fadd_rn(__fadd_rn(__fmul_rn(nx, qx), __fmul_rn(ny, qy)), __fmul_rn(nz, qz));
    Q.px = __fadd_rn(Q.px, qx);
    Q.py = __fadd_rn(Q.py, qy);
    Q.pz = __fadd_rn(Q.pz, qz);
    const float n3[3] = {nx, ny, nz};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Q.ata[3 * i + j] = acc_mul(Q.ata[3 * i + j], n3[i], n3[j], Q.fma);
    Q.atb[0] = acc_mul(Q.atb[0], nx, d, Q.fma);
    Q.atb[1] = acc_mul(Q.atb[1], ny, d, Q.fma);
    Q.atb[2] = acc_mul(Q.atb[2], nz, d, Q.fma);
}

// The regularisation, the eigen-decomposition and the solution of K crossings.
__device__ __forceinline__ void qef_finish(Qef& Q, uint32_t K, float reg, float svd_tol) {
    float* ata = Q.ata;
    float* atb = Q.atb;
    const float cnt = __uint2float_rn(K);
    const float px = __fdiv_rn(Q.px, cnt), py = __fdiv_rn(Q.py, cnt), pz = __fdiv_rn(Q.pz, cnt);
    ata[0] = __fadd_rn(ata[0], reg); ata[4] = __fadd_rn(ata[4], reg); ata[8] = __fadd_rn(ata[8], reg);
    atb[0] = acc_mul(atb[0], reg, px, Q.fma);
    atb[1] = acc_mul(atb[1], reg, py, Q.fma);
    atb[2] = acc_mul(atb[2], reg, pz, Q.fma);
    // pseudo-inverse solve: singular values of the symmetric system are |w|
    float m[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) m[i][j] = ata[3 * i + j];
    jacobi3f(m, Q.w, Q.q);
    const float smax = fmaxf(fabsf(Q.w[0]), fmaxf(fabsf(Q.w[1]), fabsf(Q.w[2])));
    const float thr = svd_tol * smax;
    unsigned keep = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) keep |= (fabsf(Q.w[i]) > thr ? 1u : 0u) << i;
    Q.keep = keep;
    float xf[3] = {0.0f, 0.0f, 0.0f};
    apply_pinv_f(Q.w, Q.q, keep, atb, xf);
    // one refinement step with a residual to twice FP32's precision (the FP32
    // eigenvectors leave an error of about cond(A) * eps; the residual recovers it)
    float r[3], dx[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = residual_ff(atb[i], ata + 3 * i, xf);
    apply_pinv_f(Q.w, Q.q, keep, r, dx);
#pragma unroll
    for (int i = 0; i < 3; ++i) Q.x[i] = double(xf[i]) + double(dx[i]);
}

// The QEF of K crossings stored as points [K, 3] and normals [K, 3].
__device__ __forceinline__ void qef_solve(const float* points, const float* normals, uint32_t K, float reg,
                                          float svd_tol, bool fma, Qef& Q) {
    qef_init(Q, fma);
    for (uint32_t k = 0; k < K; ++k)
        qef_add(Q, points[3 * k], points[3 * k + 1], points[3 * k + 2], normals[3 * k], normals[3 * k + 1],
                normals[3 * k + 2]);
    qef_finish(Q, K, reg, svd_tol);
}

// The corners of edge e (ISO_EDGE_CORNERS) from two packed immediates, 3 bits
// per corner: lanes with different edges do not serialise on a constant-memory
// load.
constexpr unsigned long long pack_corners(int end) {
    unsigned long long p = 0;
    for (int e = 0; e < 12; ++e) p |= (unsigned long long)iso_edge_corner(2 * e + end) << (3 * e);
    return p;
}
constexpr unsigned long long EDGE_CA = pack_corners(0), EDGE_CB = pack_corners(1);
__device__ __forceinline__ int edge_ca(int e) { return int((EDGE_CA >> (3 * e)) & 7ull); }
__device__ __forceinline__ int edge_cb(int e) { return int((EDGE_CB >> (3 * e)) & 7ull); }

// Crossed edges of a cell with case bits cs (ISO_EDGE_STATUS[cs]): the edges
// whose corners differ in sign.
__device__ __forceinline__ uint32_t edge_status(uint32_t cs) {
    uint32_t est = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e)
        est |= (((cs >> iso_edge_corner(2 * e)) ^ (cs >> iso_edge_corner(2 * e + 1))) & 1u) << e;
    return est;
}

// Value at corner j of a cell, selected (not indexed), so the cell stays in
// registers when j is not a constant.
__device__ __forceinline__ float corner_value(const CellCorners& cc, int j) {
    const float a = (j & 1) ? cc.v[1] : cc.v[0], b = (j & 1) ? cc.v[3] : cc.v[2];
    const float c = (j & 1) ? cc.v[5] : cc.v[4], d = (j & 1) ? cc.v[7] : cc.v[6];
    const float lo = (j & 2) ? b : a, hi = (j & 2) ? d : c;
    return (j & 4) ? hi : lo;
}

// Position of corner j = 4 dx + 2 dy + dz: each coordinate is the low or the
// high one of the cell (corner 0 or corner 7).
__device__ __forceinline__ void corner_pos(const CellCorners& cc, int j, float* q) {
    q[0] = (j & 4) ? cc.p[7][0] : cc.p[0][0];
    q[1] = (j & 2) ? cc.p[7][1] : cc.p[0][1];
    q[2] = (j & 1) ? cc.p[7][2] : cc.p[0][2];
}

// Crossing of edge e of a cell: t and the point (the reference's lerp).
__device__ __forceinline__ float edge_cross(const CellCorners& cc, float level, int e, float* p) {
    const int ca = edge_ca(e), cb = edge_cb(e);
    float pa[3], pb[3];
    corner_pos(cc, ca, pa);
    corner_pos(cc, cb, pb);
    const float t = iso::cross_t(level, corner_value(cc, ca), corner_value(cc, cb));
#pragma unroll
    for (int q = 0; q < 3; ++q) p[q] = iso::lerp1(t, pa[q], pb[q], cc.fma);
    return t;
}

Grid3 make_grid(int nx, int ny, int nz, const float* amin, const float* amax) {
    Grid3 g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.fma = iso::arith_fma();
    for (int k = 0; k < 3; ++k) {
        g.amin[k] = amin[k];
        g.asize[k] = amax[k] - amin[k];
    }
    return g;
}

unsigned blocks_for(long long n, int b) { return unsigned((n + b - 1) / b); }

}  // namespace
