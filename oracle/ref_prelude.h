/* Prelude force-included when the reference's .cu sources are compiled as
 * host C++ with Thrust's OpenMP backend (oracle/build_ref.sh).  TEST
 * INFRASTRUCTURE ONLY. */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <climits>
#include <stdexcept>
#include <functional>
#include <cuda_runtime.h>
using std::isnan;
#ifndef __CUDACC__
static inline int __popc(unsigned int x) { return __builtin_popcount(x); }
#endif
#include <thrust/sequence.h>
