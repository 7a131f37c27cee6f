/*
 * host_prelude.h -- lets a host C++ compiler build the reference's device
 * file cuda_addon/particles_kernel.cu as plain host code (TEST
 * INFRASTRUCTURE: builds oracle/_ref/libfcref_host.so, the reference's own
 * kernels run on the CPU).
 *
 *  - the CUDA execution-space and memory-space keywords become empty, so the
 *    kernels become host functions and the __constant__ parameter block a
 *    host global;
 *  - threadIdx/blockIdx/blockDim become host globals that the launch loops in
 *    refhost.cpp set before each "thread" runs;
 *  - __umul24/__mul24 are restated from their documented semantics (product
 *    of the low 24 bits);
 *  - thrust::get over a std::tuple of references stands in for Thrust's zip
 *    iterator element.
 */
#pragma once
#include <cuda_runtime.h>
#include <vector_functions.h>
#include <cmath>
#include <tuple>

#undef __device__
#undef __global__
#undef __constant__
#undef __shared__
#define __device__
#define __global__
#define __constant__
#define __shared__

typedef unsigned int uint;

static uint3 threadIdx, blockIdx;
static dim3 blockDim;

static inline unsigned int __umul24(unsigned int a, unsigned int b) {
  return (a & 0xffffffu) * (b & 0xffffffu);
}
static inline int __mul24(int a, int b) {
  int sa = (int)((unsigned)a << 8) >> 8, sb = (int)((unsigned)b << 8) >> 8;
  return (int)((unsigned)sa * (unsigned)sb);
}
static inline void __syncthreads() {}

namespace thrust {
template <int I, class T> auto &get(T &t) { return std::get<I>(t); }
}  // namespace thrust

/* the reorder kernel's dynamic shared array (blockDim + 1 entries) */
static uint fcref_shared_hash[1025];
#define sharedHash fcref_shared_hash
