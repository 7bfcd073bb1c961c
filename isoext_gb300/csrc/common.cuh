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

// Bounded spin limit for mbarrier waits: about a second of polling.
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

// Word w of the row shifted so that bit c holds the row's bit c - 1.
__device__ __forceinline__ uint32_t prev1(const uint32_t* row, int w) {
    uint32_t lo = w > 0 ? row[w - 1] : 0u;
    return __funnelshift_l(lo, row[w], 1);
}
// Word w of the row shifted so that bit c holds the row's bit c + 1.
__device__ __forceinline__ uint32_t next1(const uint32_t* row, int w, int nw) {
    uint32_t hi = (w + 1 < nw) ? row[w + 1] : 0u;
    return __funnelshift_r(row[w], hi, 1);
}
__device__ __forceinline__ uint32_t bit_at(const uint32_t* row, int c) {
    return (row[c >> 5] >> (c & 31)) & 1u;
}
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
// Warp-cooperative iteration over the set bits of a sequence of words.
//
// The warp takes 32 words at a time (one per lane), counts their set bits,
// and hands the bits out 32 at a time, so sparse bits are processed with all
// lanes busy instead of one lane per word.  get(i) returns word i (0 for
// i >= n); f(i, b) runs once per set bit b of word i, on some lane.  scratch
// points to 64 words of warp-private shared memory.
template <class Get, class F>
__device__ __forceinline__ void warp_foreach_bit(int first, int n, int stride, uint32_t* scratch,
                                                 Get get, F f) {
    const int lane = threadIdx.x & 31;
    for (int base = first; base < n; base += stride) {
        const int i = base + lane;
        const uint32_t m = i < n ? get(i) : 0u;
        const uint32_t cnt = __popc(m);
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t x = __shfl_up_sync(~0u, incl, d);
            if (lane >= d) incl += x;
        }
        const uint32_t total = __shfl_sync(~0u, incl, 31);
        if (total == 0) continue;
        scratch[lane] = m;
        scratch[32 + lane] = incl;
        __syncwarp();
        for (uint32_t k0 = 0; k0 < total; k0 += 32) {
            const uint32_t k = k0 + lane;
            if (k < total) {
                // owner lane: first lane whose inclusive count exceeds k
                int lo = 0, hi = 31;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (scratch[32 + mid] > k) hi = mid; else lo = mid + 1;
                }
                uint32_t mm = scratch[lo];
                const uint32_t before = scratch[32 + lo] - __popc(mm);
                for (uint32_t j = k - before; j; --j) mm &= mm - 1;  // drop the lower set bits
                f(base + lo, __ffs(mm) - 1);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// TMA bulk copies (cp.async.bulk, global -> shared) completing on an mbarrier.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < ISO_SPIN_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
    }
    return false;
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
