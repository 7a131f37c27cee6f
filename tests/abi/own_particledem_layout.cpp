// The same program as ref_particledem_driver.cpp, built on fcdem_i3d.h's
// own declarations of the i3d types (no reference header): links against
// libfcdem.so and prints the member offsets, which must equal those of the
// reference's types.
#include <cstddef>
#include <cstdio>

#include "fcdem_i3d.h"

typedef i3d::HashGrid<float, i3d::cpu> HG;
typedef i3d::ParticleWorld<float, i3d::cpu> PW;
typedef i3d::SimulationParameters<float> SP;

int main(int argc, char **) {
  void *entry[] = {(void *)&cuda_init, (void *)&cuda_clean,
                   (void *)static_cast<void (*)(HG &, PW &)>(&calcHash),
                   (void *)static_cast<void (*)(HG &, PW &)>(&reorderDataAndFindCellStart),
                   (void *)&evalForces, (void *)static_cast<void (*)(HG &)>(&sortParticles),
                   (void *)static_cast<void (*)(float *, float *, float, unsigned)>(
                       &integrateSystem)};
  int n = 0;
  for (void *p : entry) n += p != nullptr;
  std::printf("resolved %d of 7\n", n);
  std::printf("SP %zu %zu %zu %zu %zu %zu\n", sizeof(SP), offsetof(SP, timeStep_),
              offsetof(SP, origin_), offsetof(SP, gravity_), offsetof(SP, gridx_),
              offsetof(SP, numParticles_));
  std::printf("HG %zu %zu %zu %zu %zu %zu %zu\n", sizeof(HG), offsetof(HG, numCells_),
              offsetof(HG, hashEntries_), offsetof(HG, cellEnd_), offsetof(HG, gridx_),
              offsetof(HG, cellSize_), offsetof(HG, origin_));
  std::printf("PW %zu %zu %zu %zu\n", sizeof(PW), offsetof(PW, pos_), offsetof(PW, sortedVel_),
              offsetof(PW, size_));
  return n == 7 ? 0 : 1;
}
