/*
 * CUDA-emulation header used ONLY to compile the reference's own
 * src/kernels.cu with g++ for the CPU, so that its kernels can be executed
 * thread by thread as a checker for the oracle (oracle/ref/ref_kernels.cpp).
 * It stands in for <cuda_runtime.h> on the include path of that one build.
 *
 * A kernel "launch" is a loop over (blockIdx, threadIdx) that sets the
 * globals below and calls the __global__ function as a plain C++ function.
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <math.h>
#include <stdlib.h>

struct dim3 {
    unsigned x, y, z;
};

extern dim3 threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__
#define __host__
#define __shared__ static

inline void __syncthreads() {}

using std::abs;
using std::max;
using std::min;
