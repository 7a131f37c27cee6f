// Compiled by tests/test_reference_headers.py with the reference's own i3d
// container types (inshape3dcore/grid/uniformgrid.h, whose include guards
// make fcdem_i3d.h declare its functions on those types), linked against
// libfcdem.so: the link succeeds only if the library exports the particledem
// functions under the names a caller compiled against the reference binds
// to.  Also prints the member offsets of the three types.
#include <cstddef>
#include <cstdio>

#include "uniformgrid.h"
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
