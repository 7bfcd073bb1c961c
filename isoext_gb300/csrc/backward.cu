// Backward passes: gradients of extracted vertex positions with respect to the
// grid values (sm_103a).  Topology is integer and has no gradient: which edges
// cross, which cells are active and the faces stay fixed.  Vertex positions are
// differentiable functions of the values.
//
//   marching cubes   v = lerp(t, pa, pb), t = (level - va) / (vb - va)
//                    (src/mc/nagae.cu:52-56, include/math.cuh:77-81).  Only the
//                    edge's axis moves: dv/dt = pb - pa along it, and
//                    dt/dva = -(1 - t) / (vb - va), dt/dvb = -t / (vb - va).
//   dual contouring  x = pinv(M) r with M = sum n n^T + reg I and
//                    r = sum n (n . p) + reg mean(p) (src/dc.cu:14-65), clipped
//                    to the cell (src/dc.cu:82-99).  Implicit differentiation of
//                    M x = r gives dL/dr = lambda = pinv(M) g and
//                    dL/dM = -lambda x^T, with g zero in clipped coordinates.
//                    Per crossing this is dL/dn = lambda (n . (p - x)) + (p - x)(lambda . n)
//                    and dL/dp = n (lambda . n) + (reg / K) lambda.  Crossing
//                    points depend on the values through t, and normals taken
//                    from the grid through the cell's trilinear interpolant and
//                    its central-difference stencil (src/its.cu:170-268).
//
// Gradients are accumulated into grad_values with atomics: a grid value feeds
// several vertices.  The summation order varies between runs (FP32 rounding
// differences only).
#include <cstdint>

#include "common.cuh"
#define ISO_LUT_DECL static __constant__ const
#include "luts.h"
#include "dc_common.cuh"
#include "profile.cuh"

namespace {

__global__ void __launch_bounds__(256) mc_backward(const float* __restrict__ vals, Grid3 g, float level,
                                                   const long long* __restrict__ vedge, long long V,
                                                   const float* __restrict__ gv, float* gvals) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const long long key = vedge[i];
    const long long ia = key / 3;
    const int ax = int(key - 3 * ia);
    const long long syz = (long long)g.ny * g.nz;
    const long long step = ax == 0 ? syz : (ax == 1 ? (long long)g.nz : 1ll);
    const float va = vals[ia], vb = vals[ia + step];
    const float d = __fsub_rn(vb, va);
    if (d == 0.0f) return;  // t is the constant 0 there
    const float t = iso::cross_t(level, va, vb);
    const int c = ax == 0 ? int(ia / syz) : (ax == 1 ? int((ia / g.nz) % g.ny) : int(ia % g.nz));
    const float h = coord(g, ax, uint32_t(c + 1)) - coord(g, ax, uint32_t(c));
    const float gt = gv[3 * i + ax] * h;
    atomicAdd(gvals + ia, -gt * (1.0f - t) / d);
    atomicAdd(gvals + ia + step, -gt * t / d);
}

// Trilinear weights at t and their derivatives along each axis (corner
// j = 4x + 2y + z, the order of trilin()).
__device__ __forceinline__ void tri_weights(const float t[3], float w[8], float dw[3][8]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int bx = j >> 2, by = (j >> 1) & 1, bz = j & 1;
        const float fx = bx ? t[0] : 1.0f - t[0], fy = by ? t[1] : 1.0f - t[1], fz = bz ? t[2] : 1.0f - t[2];
        const float sx = bx ? 1.0f : -1.0f, sy = by ? 1.0f : -1.0f, sz = bz ? 1.0f : -1.0f;
        w[j] = fx * fy * fz;
        dw[0][j] = sx * fy * fz;
        dw[1][j] = fx * sy * fz;
        dw[2][j] = fx * fy * sz;
    }
}

// Gradient of the grid normal at crossing point p (cell_normal) given dL/dn:
// adds to the cell's corner values (gc) and to the point (gp).
__device__ __forceinline__ void normal_backward(const CellCorners& cc, const float* p, const float* gn, float* gp,
                                                float* gc) {
    const float eps = 0.02f;
    float cmin[3], csz[3], t[3], tin[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cmin[a] = cc.p[0][a];
        csz[a] = __fsub_rn(cc.p[7][a], cc.p[0][a]);
        const float r = __fdiv_rn(__fsub_rn(p[a], cmin[a]), csz[a]);
        t[a] = fmaxf(0.01f, fminf(0.99f, r));
        tin[a] = (r > 0.01f && r < 0.99f) ? 1.0f : 0.0f;
    }
    float d[3], den[3], fp[3], fm[3], sp[3], sm[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float tp[3] = {t[0], t[1], t[2]}, tm[3] = {t[0], t[1], t[2]};
        tp[a] = fminf(__fadd_rn(t[a], eps), 0.99f);
        tm[a] = fmaxf(__fsub_rn(t[a], eps), 0.01f);
        sp[a] = __fadd_rn(t[a], eps) < 0.99f ? 1.0f : 0.0f;
        sm[a] = __fsub_rn(t[a], eps) > 0.01f ? 1.0f : 0.0f;
        // the adjoint needs the stencil's values only to first order
        fp[a] = iso::trilin_t<false, false>(cc.v, tp[0], tp[1], tp[2]);
        fm[a] = iso::trilin_t<false, false>(cc.v, tm[0], tm[1], tm[2]);
        den[a] = __fmul_rn(__fsub_rn(tp[a], tm[a]), csz[a]);
        d[a] = __fdiv_rn(__fsub_rn(fp[a], fm[a]), den[a]);
    }
    const float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(len > 1e-8f)) return;  // the normal is the constant (0, 0, 1) there
    const float n[3] = {d[0] / len, d[1] / len, d[2] / len};
    const float ng = n[0] * gn[0] + n[1] * gn[1] + n[2] * gn[2];
    float gd[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) gd[a] = (gn[a] - n[a] * ng) / len;
    float gt[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float tp[3] = {t[0], t[1], t[2]}, tm[3] = {t[0], t[1], t[2]};
        tp[a] = fminf(t[a] + eps, 0.99f);
        tm[a] = fmaxf(t[a] - eps, 0.01f);
        float wp[8], wm[8], dwp[3][8], dwm[3][8];
        tri_weights(tp, wp, dwp);
        tri_weights(tm, wm, dwm);
        const float s = gd[a] / den[a];
#pragma unroll
        for (int j = 0; j < 8; ++j) gc[j] += s * (wp[j] - wm[j]);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float dfp = 0.0f, dfm = 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                dfp += cc.v[j] * dwp[b][j];
                dfm += cc.v[j] * dwm[b][j];
            }
            if (b == a) {
                dfp *= sp[a];
                dfm *= sm[a];
            }
            gt[b] += s * (dfp - dfm);
        }
        // the stencil's width (tp - tm) * csz changes where one side is clamped
        gt[a] -= gd[a] * d[a] / den[a] * (sp[a] - sm[a]) * csz[a];
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) gp[b] += gt[b] * tin[b] / csz[b];
}

// One thread per active cell.  The crossings, their normals and the QEF are
// recomputed in the forward's order (the same bits), then the crossings are
// walked again for the gradients; the cell's corners stay in registers (edge
// corners are selected, not indexed).
__global__ void __launch_bounds__(128) dc_backward(const float* __restrict__ vals, Grid3 g, float level,
                                                   const uint32_t* __restrict__ cell_ids,
                                                   const uint32_t* __restrict__ cell_off, long long A,
                                                   float reg, float svd_tol,
                                                   const float* __restrict__ user_normals,
                                                   const float* __restrict__ gdual, float* gvals,
                                                   float* gnormals) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    float gx[3] = {gdual[3 * a], gdual[3 * a + 1], gdual[3 * a + 2]};
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
    const uint32_t k0 = cell_off[a];
    // the forward again: the QEF of the crossings in edge order
    Qef Q;
    qef_init(Q, g.fma);
    uint32_t K = 0;
#pragma unroll 1
    for (uint32_t em = est; em; em &= em - 1, ++K) {
        const int e = __ffs(em) - 1;
        float p[3], n[3];
        edge_cross(cc, level, e, p);
        if (user_normals) {
#pragma unroll
            for (int q = 0; q < 3; ++q) n[q] = user_normals[3ll * (k0 + K) + q];
        } else {
            cell_normal(cc, p, n);
        }
        qef_add(Q, p[0], p[1], p[2], n[0], n[1], n[2]);
    }
    qef_finish(Q, K, reg, svd_tol);
    const int ci[3] = {cx, cy, cz};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float lo = coord(g, q, uint32_t(ci[q])), hi = coord(g, q, uint32_t(ci[q] + 1));
        const float xf = float(Q.x[q]);
        if (xf < lo || xf > hi) gx[q] = 0.0f;  // clipped: the output does not move
    }
    if (gx[0] == 0.0f && gx[1] == 0.0f && gx[2] == 0.0f) return;
    float l[3] = {0.0f, 0.0f, 0.0f};
    apply_pinv_f(Q.w, Q.q, Q.keep, gx, l);  // lambda = pinv(M) g
    const float rk = reg / float(K);
    float gc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t k = 0;
#pragma unroll 1
    for (uint32_t em = est; em; em &= em - 1, ++k) {
        const int e = __ffs(em) - 1;
        float p[3], n[3];
        const float t = edge_cross(cc, level, e, p);
        if (user_normals) {
#pragma unroll
            for (int q = 0; q < 3; ++q) n[q] = user_normals[3ll * (k0 + k) + q];
        } else {
            cell_normal(cc, p, n);
        }
        float u[3], gn[3], gp[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) u[q] = float(double(p[q]) - Q.x[q]);
        const float ln = l[0] * n[0] + l[1] * n[1] + l[2] * n[2];
        const float nu = n[0] * u[0] + n[1] * u[1] + n[2] * u[2];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            gn[q] = l[q] * nu + u[q] * ln;
            gp[q] = n[q] * ln + rk * l[q];
        }
        if (user_normals) {
            if (gnormals) {
#pragma unroll
                for (int q = 0; q < 3; ++q) gnormals[3ll * (k0 + k) + q] = gn[q];
            }
        } else {
            normal_backward(cc, p, gn, gp, gc);
        }
        // through the crossing's t to the edge's two corner values
        const int ca = edge_ca(e), cb = edge_cb(e);
        const float d = corner_value(cc, cb) - corner_value(cc, ca);
        if (d == 0.0f) continue;
        float pa[3], pb[3];
        corner_pos(cc, ca, pa);
        corner_pos(cc, cb, pb);
        float gt = 0.0f;
#pragma unroll
        for (int q = 0; q < 3; ++q) gt += gp[q] * (pb[q] - pa[q]);
        const float ga = -(gt * (1.0f - t) / d), gb = -(gt * t / d);
#pragma unroll
        for (int j = 0; j < 8; ++j) gc[j] += (j == ca ? ga : 0.0f) + (j == cb ? gb : 0.0f);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (gc[j] == 0.0f) continue;
        const int x = cx + (j >> 2), y = cy + ((j >> 1) & 1), z = cz + (j & 1);
        atomicAdd(gvals + ((long long)x * g.ny + y) * g.nz + z, gc[j]);
    }
}

// grad_dual[src[i]] = grad_vertices[i]: each dual vertex is the source of at
// most one welded vertex.
__global__ void dc_scatter_src(const int* __restrict__ src, long long V, const float* __restrict__ gv,
                               float* __restrict__ gdual) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    const long long a = src[i];
    gdual[3 * a] = gv[3 * i];
    gdual[3 * a + 1] = gv[3 * i + 1];
    gdual[3 * a + 2] = gv[3 * i + 2];
}

}  // namespace

extern "C" {

int iso_mc_backward(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                    float level, const long long* vertex_edges, long long V, const float* grad_vertices,
                    float* grad_values, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (V < 0 || nx < 2 || ny < 2 || nz < 2 || !aabb_min || !aabb_max) return iso::fail_code(ISO_ERR_ARG);
    if (V == 0) return 0;
    if (!values || !vertex_edges || !grad_vertices || !grad_values) return iso::fail_code(ISO_ERR_ARG);
    const Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    iso::ProfScope ps("mc_backward", st);
    mc_backward<<<blocks_for(V, 256), 256, 0, st>>>(values, g, level, vertex_edges, V, grad_vertices, grad_values);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_backward(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                    float level, const int* cell_ids, const int* cell_offsets, long long A, float reg,
                    float svd_tol, const float* normals, const float* grad_dual, float* grad_values,
                    float* grad_normals, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A < 0 || nx < 2 || ny < 2 || nz < 2 || !aabb_min || !aabb_max) return iso::fail_code(ISO_ERR_ARG);
    if (A == 0) return 0;
    if (!values || !cell_ids || !cell_offsets || !grad_dual || !grad_values) return iso::fail_code(ISO_ERR_ARG);
    const Grid3 g = make_grid(nx, ny, nz, aabb_min, aabb_max);
    iso::ProfScope ps("dc_backward", st);
    dc_backward<<<blocks_for(A, 128), 128, 0, st>>>(values, g, level, reinterpret_cast<const uint32_t*>(cell_ids),
                                                    reinterpret_cast<const uint32_t*>(cell_offsets), A, reg,
                                                    svd_tol, normals, grad_dual, grad_values, grad_normals);
    return cudaGetLastError() == cudaSuccess ? 0 : iso::fail_code(ISO_ERR_CUDA);
}

int iso_dc_backward_src(const float* values, int nx, int ny, int nz, const float* aabb_min, const float* aabb_max,
                        float level, const int* cell_ids, const int* cell_offsets, long long A, float reg,
                        float svd_tol, const int* vertex_source, long long V, const float* grad_vertices,
                        float* grad_dual_ws, float* grad_values, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (A < 0 || V < 0 || nx < 2 || ny < 2 || nz < 2 || !aabb_min || !aabb_max || !grad_values) return iso::fail_code(ISO_ERR_ARG);
    if (cudaMemsetAsync(grad_values, 0, size_t(nx) * ny * nz * sizeof(float), st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    if (A == 0 || V == 0) return 0;
    if (!values || !cell_ids || !cell_offsets || !vertex_source || !grad_vertices || !grad_dual_ws) return iso::fail_code(ISO_ERR_ARG);
    if (cudaMemsetAsync(grad_dual_ws, 0, size_t(A) * 3 * sizeof(float), st) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
    {
        iso::ProfScope ps("dc_backward", st);
        dc_scatter_src<<<blocks_for(V, 256), 256, 0, st>>>(vertex_source, V, grad_vertices, grad_dual_ws);
    }
    return iso_dc_backward(values, nx, ny, nz, aabb_min, aabb_max, level, cell_ids, cell_offsets, A, reg, svd_tol,
                           nullptr, grad_dual_ws, grad_values, nullptr, stream);
}

}  // extern "C"
