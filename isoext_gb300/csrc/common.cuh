// Shared device helpers for the iso-surface kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

// Error codes written to the device status word and returned by the C ABI.
enum IsoStatus : int {
    ISO_OK = 0,
    ISO_ERR_ARG = 1,          // invalid argument (host check)
    ISO_ERR_CUDA = 2,         // CUDA runtime error
    ISO_ERR_TIMEOUT = 3,      // a bounded device wait ran out
    ISO_ERR_LOOKUP = 4,       // a face referenced a vertex that was not emitted
    ISO_ERR_WORKSPACE = 5,    // workspace too small
    ISO_ERR_OVERFLOW = 6,     // output capacity exceeded (counts are still exact)
};

// Polls before a bounded device wait gives up (with a sleep between polls: a
// few seconds at most).
#define ISO_SPIN_LIMIT (1u << 26)

namespace iso {

// ---------------------------------------------------------------------------
// The reference's FP32 expressions, in two readings selected by `fma`:
//   true  -- what nvcc's default FMA contraction (-fmad=true) makes of isoext's
//            source, i.e. the arithmetic of its CUDA build, which is what isoext
//            users run.  The fused forms below were measured on sm_103a with
//            nvcc 13.0: a restatement of the source compiled with default flags
//            gives these bits on every input tried (tests/nvcc_expr.cu).
//   false -- every operation rounded on its own: the source read literally,
//            which is what its host build (x86, no FMA) computes.
// Every other operation is explicitly rounded, so neither reading depends on
// how this library itself is compiled.

// Grid point coordinate: amin + (i / (float)(n - 1)) * size
// (include/utils.cuh:62-80, get_vtx_pos_op); nvcc fuses the multiply-add.
__device__ __forceinline__ float grid_coord(uint32_t i, uint32_t n, float amin, float size, bool fma) {
    const float f = __fdiv_rn(__uint2float_rn(i), __uint2float_rn(n - 1u));
    return fma ? __fmaf_rn(f, size, amin) : __fadd_rn(amin, __fmul_rn(f, size));
}

// Edge crossing parameter t = (level - va) / (vb - va), 0 when vb == va
// (src/mc/nagae.cu:52-53).  Nothing to fuse.
__device__ __forceinline__ float cross_t(float level, float va, float vb) {
    const float d = __fsub_rn(vb, va);
    return d != 0.0f ? __fdiv_rn(__fsub_rn(level, va), d) : 0.0f;
}

// x * ox + y * oy, the shape of lerp and of each trilinear step.  nvcc fuses
// the first product (fma(x, ox, y * oy)); `swap` is the other fusion,
// fma(y, oy, x * ox), which it picks for some steps of the normal stencil.
__device__ __forceinline__ float blend2(float x, float ox, float y, float oy, bool fma, bool swap = false) {
    if (!fma) return __fadd_rn(__fmul_rn(x, ox), __fmul_rn(y, oy));
    return swap ? __fmaf_rn(y, oy, __fmul_rn(x, ox)) : __fmaf_rn(x, ox, __fmul_rn(y, oy));
}

// lerp(t, a, b) = (1 - t) * a + t * b per component (include/math.cuh:77-81).
__device__ __forceinline__ float lerp1(float t, float a, float b, bool fma) {
    return blend2(__fsub_rn(1.0f, t), a, t, b, fma);
}

// |d| = sqrt(d.x*d.x + d.y*d.y + d.z*d.z) (include/math.cuh, norm and dot);
// nvcc: sqrt(fma(z, z, fma(x, x, y * y))).
__device__ __forceinline__ float norm3f(float x, float y, float z, bool fma) {
    if (!fma) return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
    return __fsqrt_rn(__fmaf_rn(z, z, __fmaf_rn(x, x, __fmul_rn(y, y))));
}

// Trilinear interpolation of corner values cv (corner j = 4x + 2y + z) at t
// (src/its.cu:170-184): along z, then y, then x.  kSwapLowZ: the nvcc fusion
// of the two x = 0 steps along z is the swapped one (see stencil_normal).
template <bool F, bool kSwapLowZ>
__device__ __forceinline__ float trilin_t(const float* cv, float tx, float ty, float tz) {
    const float oz = __fsub_rn(1.0f, tz), oy = __fsub_rn(1.0f, ty), ox = __fsub_rn(1.0f, tx);
    const float c00 = blend2(cv[0], oz, cv[1], tz, F, kSwapLowZ);
    const float c01 = blend2(cv[2], oz, cv[3], tz, F, kSwapLowZ);
    const float c10 = blend2(cv[4], oz, cv[5], tz, F);
    const float c11 = blend2(cv[6], oz, cv[7], tz, F);
    const float c0 = blend2(c00, oy, c01, ty, F);
    const float c1 = blend2(c10, oy, c11, ty, F);
    return blend2(c0, ox, c1, tx, F);
}

// fmaxf(0.01, fminf(0.99, d / csz)), the stencil's clamped cell coordinate,
// with the division only where its result can lie inside (0.01, 0.99).  For
// csz >= 1e-30 (so that 0.009 csz is a normal float, rounded by at most 2^-24
// of itself): d <= fl(0.009 csz) makes d / csz < 0.0091 before rounding, so
// the rounded quotient is below 0.01 and the clamp gives 0.01; d >=
// fl(0.991 csz) makes it above 0.9909, and the clamp gives 0.99.  On the two
// axes across a crossing's edge, d is within a few ulps of 0 or of csz, so
// those coordinates need no division.
__device__ __forceinline__ float clamp_cell_t(float d, float csz) {
    if (csz >= 1e-30f) {
        if (d <= __fmul_rn(0.009f, csz)) return 0.01f;
        if (d >= __fmul_rn(0.991f, csz)) return 0.99f;
    }
    return fmaxf(0.01f, fminf(0.99f, __fdiv_rn(d, csz)));
}

template <bool F>
__device__ __forceinline__ void stencil_normal_t(const float* v, const float* lo, const float* hi, const float* p,
                                                 float* n) {
    float csz[3], t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        csz[a] = __fsub_rn(hi[a], lo[a]);
        t[a] = clamp_cell_t(__fsub_rn(p[a], lo[a]), csz[a]);
    }
    const float eps = 0.02f;
    const float xp = fminf(__fadd_rn(t[0], eps), 0.99f), xm = fmaxf(__fsub_rn(t[0], eps), 0.01f);
    const float yp = fminf(__fadd_rn(t[1], eps), 0.99f), ym = fmaxf(__fsub_rn(t[1], eps), 0.01f);
    const float zp = fminf(__fadd_rn(t[2], eps), 0.99f), zm = fmaxf(__fsub_rn(t[2], eps), 0.01f);
    // the four samples at the crossing's own z share their steps along z; for
    // those nvcc swaps the fusion of the x = 0 steps
    const float dx = __fdiv_rn(__fsub_rn(trilin_t<F, true>(v, xp, t[1], t[2]), trilin_t<F, true>(v, xm, t[1], t[2])),
                               __fmul_rn(__fsub_rn(xp, xm), csz[0]));
    const float dy = __fdiv_rn(__fsub_rn(trilin_t<F, true>(v, t[0], yp, t[2]), trilin_t<F, true>(v, t[0], ym, t[2])),
                               __fmul_rn(__fsub_rn(yp, ym), csz[1]));
    const float dz = __fdiv_rn(__fsub_rn(trilin_t<F, false>(v, t[0], t[1], zp), trilin_t<F, false>(v, t[0], t[1], zm)),
                               __fmul_rn(__fsub_rn(zp, zm), csz[2]));
    const float len = norm3f(dx, dy, dz, F);
    if (len > 1e-8f) {
        n[0] = __fdiv_rn(dx, len);
        n[1] = __fdiv_rn(dy, len);
        n[2] = __fdiv_rn(dz, len);
    } else {
        n[0] = 0.0f; n[1] = 0.0f; n[2] = 1.0f;
    }
}

// Normal at crossing point p of the cell with corner values v and corners lo
// (corner 0) and hi (corner 7): central differences of the trilinear
// interpolant at +-0.02 cell units, clamped to [0.01, 0.99], normalised
// (src/its.cu:186-268).
__device__ __forceinline__ void stencil_normal(const float* v, const float* lo, const float* hi, const float* p,
                                               float* n, bool fma) {
    if (fma) stencil_normal_t<true>(v, lo, hi, p, n);
    else stencil_normal_t<false>(v, lo, hi, p, n);
}

// Case bit of a corner: (v - level < 0) (include/utils.cuh:96-99).
__device__ __forceinline__ bool below(float v, float level) { return __fsub_rn(v, level) < 0.0f; }

// ---------------------------------------------------------------------------
// Bit helpers on rows of 32-bit words indexed by column c (bit c & 31 of word c >> 5).

// Mask of bits [lo, hi] (inclusive, in column units) within word w.
__device__ __forceinline__ uint32_t range_mask(int w, int lo, int hi) {
    int a = lo - 32 * w, b = hi - 32 * w;
    if (b < 0 || a > 31 || hi < lo) return 0u;
    if (a < 0) a = 0;
    if (b > 31) b = 31;
    uint32_t top = (b == 31) ? 0xffffffffu : ((2u << b) - 1u);
    return top & ~((1u << a) - 1u);
}

// ---------------------------------------------------------------------------
// Exact-position welds compare positions as bit patterns with -0 read as +0
// (float equality, except that NaNs of one pattern match each other).

__device__ __forceinline__ uint32_t pos_bits(float f) { return __float_as_uint(f == 0.0f ? 0.0f : f); }
__device__ __forceinline__ uint32_t pos_hash(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch: a kernel launched with launch_pdl may start
// while the previous kernel on its stream finishes; grid_wait() blocks until
// that kernel has completed and its writes are visible.  Every kernel launched
// this way calls it before touching memory the previous kernels use.

__device__ __forceinline__ void grid_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... Params, typename... Args>
cudaError_t launch_pdl(void (*kernel)(Params...), unsigned grid, unsigned block, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

// ---------------------------------------------------------------------------
// Launch parameters the autotuner may change (process-wide; iso_tune_set).

enum TuneKey { TUNE_MC_SIGN_CTAS = 0, TUNE_DC_CELL_THREADS = 1, TUNE_MC_COUNT_THREADS = 2, TUNE_KEYS = 3 };
int tune_get(int key);

// Arithmetic reading for the next launches (iso_set_arith; process-wide):
// true = the reference's CUDA build (fused), false = its host build.
bool arith_fma();

// An entry point's failure: sets the message iso_last_error returns on this
// thread to the plain meaning of `code` (with CUDA's error text for
// ISO_ERR_CUDA) and returns `code`.
int fail_code(int code);

}  // namespace iso
