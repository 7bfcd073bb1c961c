// Bulk copy by the SMs.  On a Grace-Blackwell node the GPU reads pinned host
// memory coherently over NVLink-C2C; a kernel with many 16-byte loads in flight
// per thread moves a host buffer into HBM faster than one copy-engine transfer.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "profile.cuh"

namespace {

constexpr int COPY_THREADS = 256;
constexpr int COPY_UNROLL = 8;

__global__ void __launch_bounds__(COPY_THREADS) copy16(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                       long long n) {
    const long long stride = (long long)gridDim.x * COPY_THREADS;
    long long i = (long long)blockIdx.x * COPY_THREADS + threadIdx.x;
    for (; i + (COPY_UNROLL - 1) * stride < n; i += COPY_UNROLL * stride) {
        uint4 v[COPY_UNROLL];
#pragma unroll
        for (int u = 0; u < COPY_UNROLL; ++u) v[u] = src[i + u * stride];
#pragma unroll
        for (int u = 0; u < COPY_UNROLL; ++u) dst[i + u * stride] = v[u];
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

__global__ void copy1(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

}  // namespace

extern "C" {

// Copy `bytes` from src to dst on the stream with a kernel.  src and dst are
// device-accessible: device memory, or pinned host memory (which the GPU
// addresses directly under unified addressing).  No counterpart in isoext.
int iso_copy(void* dst, const void* src, long long bytes, void* stream) {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (bytes < 0 || (bytes && (!dst || !src))) return ISO_ERR_ARG;
    if (bytes == 0) return 0;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    iso::ProfScope ps("copy", st);
    const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0;
    long long head = 0;
    if (aligned) {
        const long long n16 = bytes / 16;
        if (n16) {
            const long long want = (n16 + COPY_THREADS - 1) / COPY_THREADS;
            const long long grid = std::max<long long>(1, std::min<long long>(want, (long long)sms * 8));
            copy16<<<unsigned(grid), COPY_THREADS, 0, st>>>(reinterpret_cast<const uint4*>(src),
                                                            reinterpret_cast<uint4*>(dst), n16);
        }
        head = n16 * 16;
    }
    const long long rest = bytes - head;
    if (rest > 0) {
        if (!aligned && rest > (1ll << 20)) return ISO_ERR_ARG;  // only small unaligned copies
        copy1<<<unsigned((rest + 255) / 256), 256, 0, st>>>(reinterpret_cast<const uint8_t*>(src) + head,
                                                           reinterpret_cast<uint8_t*>(dst) + head, rest);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : ISO_ERR_CUDA;
}

}  // extern "C"
