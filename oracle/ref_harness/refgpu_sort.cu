/*
 * refgpu_sort.cu -- TEST INFRASTRUCTURE.  The reference's sort stage as its
 * launch glue issues it (cuda_addon/particleSystem.cu:265-270):
 * thrust::sort_by_key over the device arrays of hashes and indices, on the
 * legacy default stream, with Thrust's own temporary allocation per call.
 * Together with refgpu_loader.cpp (the other stages' glue over the
 * reference's own kernels) this times the reference's GPU step.
 */
#include <thrust/device_ptr.h>
#include <thrust/sort.h>

extern "C" int fcrefgpu_sort_by_key(unsigned *keys, unsigned *vals, unsigned n) {
  try {
    thrust::sort_by_key(thrust::device_ptr<unsigned>(keys),
                        thrust::device_ptr<unsigned>(keys + n),
                        thrust::device_ptr<unsigned>(vals));
  } catch (...) {
    return 1;
  }
  return 0;
}
