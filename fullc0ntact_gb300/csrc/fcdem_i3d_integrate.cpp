// fcdem_i3d_integrate.cpp -- the C++-linkage integrateSystem of the
// particledem interface (cuda_addon/particledem.cu:449-460).  It has the
// argument list of the extern "C" integrateSystem of the particleSystem
// interface, so it is defined in a translation unit that does not see
// fcdem.h.
#include "../../include/fcdem_i3d.h"

namespace fcdem {
void i3dIntegrate(float *pos, float *vel, float dt, unsigned n);  // fcdem_i3d.cu
}

void integrateSystem(float *pos, float *vel, float deltaTime, unsigned int numParticles) {
  fcdem::i3dIntegrate(pos, vel, deltaTime, numParticles);
}
