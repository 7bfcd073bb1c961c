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
// Exact FP32 arithmetic.  Every operation is rounded on its own (no FMA
// contraction): this is the reference's source read literally, and what its
// host build computes.

// Grid point coordinate: amin + (i / (float)(n - 1)) * size
// (include/utils.cuh:62-80, get_vtx_pos_op).
__device__ __forceinline__ float grid_coord(uint32_t i, uint32_t n, float amin, float size) {
    float f = __fdiv_rn(__uint2float_rn(i), __uint2float_rn(n - 1u));
    return __fadd_rn(amin, __fmul_rn(f, size));
}

// Edge crossing parameter t = (level - va) / (vb - va), 0 when vb == va
// (src/mc/nagae.cu:52-53).
__device__ __forceinline__ float cross_t(float level, float va, float vb) {
    float d = __fsub_rn(vb, va);
    return d != 0.0f ? __fdiv_rn(__fsub_rn(level, va), d) : 0.0f;
}

// lerp(t, a, b) = (1 - t) * a + t * b per component (include/math.cuh:77-81).
__device__ __forceinline__ float lerp1(float t, float a, float b) {
    return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, t), a), __fmul_rn(t, b));
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

enum TuneKey { TUNE_MC_SIGN_CTAS = 0, TUNE_DC_CELL_THREADS = 1, TUNE_KEYS = 2 };
int tune_get(int key);

}  // namespace iso
