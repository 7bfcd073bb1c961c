// Kernel timing hook: while enabled, every launch the library makes is
// bracketed by CUDA events on its stream, so a benchmark can read per-kernel
// device time without a profiler.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace {
struct Rec {
    const char* name;
    cudaEvent_t a, b;
    int kernels;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

namespace iso {
ProfScope::ProfScope(const char* name, cudaStream_t st, int kernels)
    : name_(name), st_(st), a_(nullptr), kernels_(kernels) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_on) return;
    a_ = get_event();
    cudaEventRecord(a_, st_);
}
ProfScope::~ProfScope() {
    if (!a_) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t b = get_event();
    cudaEventRecord(b, st_);
    g_recs.push_back({name_, a_, b, kernels_});
}
}  // namespace iso

extern "C" {

int iso_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = on != 0;
    return ISO_OK;
}

void iso_profile_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& r : g_recs) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
}

int iso_profile_read(const char* kernel, long long* launches, double* total_ms) {
    std::lock_guard<std::mutex> lk(g_mu);
    long long n = 0;
    double t = 0;
    for (auto& r : g_recs) {
        if (kernel && std::strcmp(kernel, r.name) != 0) continue;
        if (cudaEventSynchronize(r.b) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
        float ms = 0;
        if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) return iso::fail_code(ISO_ERR_CUDA);
        ++n;
        t += ms;
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = t;
    return ISO_OK;
}

int iso_profile_kernels(const char* kernel, long long* kernels) {
    if (!kernels) return iso::fail_code(ISO_ERR_ARG);
    std::lock_guard<std::mutex> lk(g_mu);
    long long n = 0;
    for (auto& r : g_recs)
        if (!kernel || std::strcmp(kernel, r.name) == 0) n += r.kernels;
    *kernels = n;
    return ISO_OK;
}

}  // extern "C"
