// Compiled by tests/test_reference_headers.py against the reference's own
// C interface headers (cuda_addon/particles_kernel.cuh, particleSystem.cuh)
// and this library's fcdem.h in one translation unit: the compiler rejects
// any extern "C" declaration of fcdem.h that differs from the reference's.
// Linked against libfcdem.so; running it resolves every entry point (no GPU
// call is made).
#include <cstdio>

#include "particles_kernel.cuh"
#include "particleSystem.cuh"
#include "fcdem.h"

static_assert(sizeof(SimParams) == 104, "the reference's SimParams");

int main() {
  void *entry[] = {
      (void *)&cudaInit, (void *)&allocateArray, (void *)&freeArray, (void *)&threadSync,
      (void *)&copyArrayFromDevice, (void *)&copyArrayToDevice, (void *)&registerGLBufferObject,
      (void *)&unregisterGLBufferObject, (void *)&mapGLBufferObject,
      (void *)&unmapGLBufferObject, (void *)&setParameters, (void *)&integrateSystem,
      (void *)&calcHash, (void *)&reorderDataAndFindCellStart, (void *)&collide,
      (void *)&sortParticles};
  int n = 0;
  for (void *p : entry) n += p != nullptr;
  std::printf("resolved %d of %d\n", n, (int)(sizeof(entry) / sizeof(entry[0])));
  return n == (int)(sizeof(entry) / sizeof(entry[0])) ? 0 : 1;
}
