/*
 * Host-compilation shim for the reference's CUDA kernel sources.
 *
 * TEST INFRASTRUCTURE ONLY. It lets g++ compile the reference kernel files
 * (every kernels/*.cu file under src/solvers/NavierStokes) unchanged, as plain C++ functions,
 * so that oracle/ref_harness.cpp can run every "thread" of a launch serially on
 * the CPU and produce golden vectors. Nothing in the product includes it.
 *
 * __global__/__device__ become nothing; threadIdx/blockIdx/blockDim become
 * thread-local globals that the harness sets before each call.
 */
#pragma once
#include <math.h>
#include <stdlib.h>
#include <cmath>
#include <cstdlib>
using std::abs;

struct ref_dim3 { unsigned int x, y, z; };
extern thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__
#define __host__
#define __shared__ static
