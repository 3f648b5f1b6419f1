// shim.h -- compile device kernel sources as host C++ for CPU checks.
//
// The CUDA headers give the vector types; each kernel call is made once per
// (block, thread) index by the check, with blockIdx/threadIdx/blockDim set
// by hand.  Shared arrays become static, so a check must run every thread
// of a block that fills one before any thread that reads it.
#ifndef CY_HOST_SHIM_H
#define CY_HOST_SHIM_H
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
using std::isfinite;
using std::min;
using std::max;
static inline int __float2int_rz(float v) { return static_cast<int>(v); }
static inline long long __float2ll_rn(float v) { return llrintf(v); }
extern "C" inline float __powf(float a, float b) { return powf(a, b); }
#define __launch_bounds__(x)
#undef __shared__
#define __shared__ static
static uint3 threadIdx, blockIdx;
static dim3 blockDim;
static inline void __syncthreads() {}
#endif
