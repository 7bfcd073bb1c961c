// RAII timing scope used around each kernel launch (see profile.cu); kernels:
// how many kernels the scope launches.
#pragma once
#include <cuda_runtime.h>

namespace iso {
class ProfScope {
  public:
    ProfScope(const char* name, cudaStream_t st, int kernels = 1);
    ~ProfScope();
    ProfScope(const ProfScope&) = delete;
    ProfScope& operator=(const ProfScope&) = delete;

  private:
    const char* name_;
    cudaStream_t st_;
    cudaEvent_t a_;
    int kernels_;
};
}  // namespace iso
