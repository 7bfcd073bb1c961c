// Decoupled look-back over tiles (single-pass prefix sums across CTAs).
//
// A tile's state word is flag << 62 | a << 31 | b (two sums < 2^31): flag 1 =
// the tile's own aggregate, 2 = its inclusive prefix, 0 = not yet published.
// Tiles take their index from a ticket counter in the order their CTAs start,
// so a tile only ever waits on tiles whose CTAs are already running.  Every
// wait is bounded: on a timeout the status is set and the prefix is wrong (the
// host sees the status).
#pragma once

#include <cstdint>

#include "common.cuh"

namespace {

constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62;
constexpr unsigned long long LB_MASK31 = 0x7fffffffull;

__device__ __forceinline__ unsigned long long lb_pack(unsigned long long flag, unsigned long long v,
                                                      unsigned long long f) {
    return flag | (min(v, LB_MASK31) << 31) | min(f, LB_MASK31);
}

// Exclusive (a, b) prefix of tile seg; run by one full warp after the tile's
// aggregate is published.
__device__ __forceinline__ void look_back(volatile unsigned long long* state, uint32_t seg, unsigned long long& ev,
                          unsigned long long& ef, int* status, uint32_t limit = ISO_SPIN_LIMIT) {
    const int lane = threadIdx.x & 31;
    ev = 0;
    ef = 0;
    long long j = (long long)seg - 1 - lane;
    while (true) {
        unsigned long long st = LB_INC;  // before tile 0: inclusive zero
        if (j >= 0) {
            uint32_t spins = 0;
            do {
                st = state[j];
                if ((st >> 62) != 0) break;
                if (++spins > limit) {
                    atomicCAS(status, 0, int(ISO_ERR_TIMEOUT));
                    st = LB_INC;
                    break;
                }
                __nanosleep(20);
            } while (true);
        }
        const uint32_t inc = __ballot_sync(~0u, (st >> 62) == 2);
        // lanes up to and including the nearest inclusive state contribute
        const int stop = inc ? __ffs(inc) - 1 : 31;
        unsigned long long v = lane <= stop ? (st >> 31) & LB_MASK31 : 0ull;
        unsigned long long f = lane <= stop ? st & LB_MASK31 : 0ull;
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) {
            v += __shfl_xor_sync(~0u, v, d);
            f += __shfl_xor_sync(~0u, f, d);
        }
        ev += v;
        ef += f;
        if (inc) break;
        j -= 32;
    }
}

// One full warp: publish tile `tile`'s aggregate (a, b), look back, publish the
// inclusive prefix.  (ea, eb) <- the exclusive prefix, on every lane.
__device__ __forceinline__ void lb_tile(unsigned long long* state, uint32_t tile, unsigned long long a,
                                        unsigned long long b, unsigned long long& ea, unsigned long long& eb,
                                        int* status) {
    const bool lead = (threadIdx.x & 31) == 0;
    ea = 0;
    eb = 0;
    if (tile == 0) {
        if (lead) atomicExch(state, lb_pack(LB_INC, a, b));
        return;
    }
    if (lead) atomicExch(state + tile, lb_pack(LB_AGG, a, b));
    look_back(state, tile, ea, eb, status);
    if (lead) atomicExch(state + tile, lb_pack(LB_INC, ea + a, eb + b));
}

}  // namespace
