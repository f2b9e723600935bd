// CPU stand-in for <cuda_runtime.h>, used only to compile the reference's
// device-code header (rSGDLM/src/kernel_functions.cuh) as plain C++ so that its
// kernels can be executed on the host by oracle/ref_driver.cpp.  Test
// infrastructure; nothing here is part of the product.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned x_ = 1, unsigned y_ = 1, unsigned z_ = 1) : x(x_), y(y_), z(z_) {}
};

extern thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

// Barrier of the emulated block: yields to the block scheduler (ref_driver.cpp).
void __syncthreads();
unsigned int atomicAdd(unsigned int *addr, unsigned int val);

using std::abs;
using std::exp;
using std::fabs;
using std::isinf;
using std::isnan;
using std::log;
using std::sqrt;
