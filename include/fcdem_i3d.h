/*
 * fcdem_i3d.h -- the particledem C++ interface of the GB300 particle-DEM
 * step: the functions of cuda_addon/particledem.cuh:11-26 on the container
 * types of inshape3dcore/grid/uniformgrid.h:470-589
 * (i3d::SimulationParameters<T>, i3d::HashGrid<T, memory>,
 * i3d::ParticleWorld<T, memory>) and inshape3dcore/fcdefines.hpp (i3d::mem).
 *
 * These are C++ functions: libfcdem.so exports them under the mangled names
 * a caller compiled against the reference's headers binds to, so host code
 * written for the reference's particledem path links against it unchanged.
 * When the reference's own headers have been included first (their include
 * guards are defined), their type definitions are used; otherwise this
 * header declares the same types with the same members in the same order
 * (layout-compatible; no Eigen needed).
 *
 * Like the reference's particleSystem.cuh and particledem.cuh, this header
 * and fcdem.h declare integrateSystem with different linkage (here C++,
 * there extern "C"); a translation unit includes one of the two.
 *
 * Semantics (cuda_addon/particledem.cu:81-460):
 *   - cuda_init: sets hg's cell size to the particle diameter, its origin and
 *     grid from *pw.params_, allocates the device arrays of hg (hg.size_
 *     entries, hg.numCells_ cells) and pw (pw.size_ particles, 4 floats
 *     each), stores their device addresses in hg and pw, sets `params` to a
 *     device copy of *pw.params_, and fills pw.pos_/pw.vel_ with the jittered
 *     lattice of particledem.cu:47-75 (srand(1973), rand()).  The contact
 *     parameters are taken from *pw.params_ here, once, as the reference's
 *     device copy is.
 *   - calcHash, sortParticles, reorderDataAndFindCellStart (cellStart and
 *     cellEnd of empty cells 0xffffffff) and evalForces (newVel = pw.vel_,
 *     no collider sphere) work on the device arrays recorded in hg and pw,
 *     with the grid of hg;
 *   - integrateSystem: the integrate of particledem.cu:412-460 in the
 *     [-1, 1]^3 box with the parameters taken at cuda_init;
 *   - cuda_clean frees the device copy of the parameters.
 * Errors are recorded for fcdemGetLastError() (fcdem.h); nothing exits.
 */
#ifndef FCDEM_I3D_H
#define FCDEM_I3D_H

#ifdef __cplusplus

#ifndef FCDEFINES_HPP_QHC1XYN6
namespace i3d {
enum mem { cpu, gpu, unified };
}  // namespace i3d
#endif

#ifndef VECTOR3_H_FLUCNCYE
namespace i3d {
template <class T>
class Vector3 {
 public:
  T x, y, z;
};
}  // namespace i3d
#endif

#ifndef UNIFORMGRID_H
namespace i3d {

/* uniformgrid.h:470-492 */
template <typename T>
class SimulationParameters {
 public:
  T spring_;
  T damping_;
  T shear_;
  T attraction_;
  T boundaryDamping_;
  T globalDamping_;
  T particleRadius_;
  T timeStep_;
  Vector3<T> origin_;
  Vector3<T> cellSize_;
  Vector3<T> gravity_;
  unsigned int gridx_, gridy_, gridz_;
  unsigned int numParticles_;
};

/* uniformgrid.h:494-535 */
template <typename T, int memory>
class HashGrid {
 public:
  unsigned int size_;
  unsigned int numCells_;
  unsigned int *hashEntries_;
  unsigned int *particleIndices_;
  unsigned int *cellStart_;
  unsigned int *cellEnd_;
  unsigned int gridx_;
  unsigned int gridy_;
  unsigned int gridz_;
  Vector3<T> cellSize_;
  Vector3<T> origin_;
};

/* uniformgrid.h:537-577 */
template <typename T, int memory>
class ParticleWorld {
 public:
  SimulationParameters<T> *params_;
  T *pos_;
  T *vel_;
  T *sortedPos_;
  T *sortedVel_;
  int size_;
};

}  // namespace i3d
#endif /* UNIFORMGRID_H */

/* particledem.cuh:11-26 */
void cuda_init(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw,
               i3d::SimulationParameters<float> *&params);
void cuda_clean();
void calcHash(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw);
void reorderDataAndFindCellStart(i3d::HashGrid<float, i3d::cpu> &hg,
                                 i3d::ParticleWorld<float, i3d::cpu> &pw);
void evalForces(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw);
void sortParticles(i3d::HashGrid<float, i3d::cpu> &hg);
#ifndef FCDEM_I3D_NO_INTEGRATE_DECL
void integrateSystem(float *pos, float *vel, float deltaTime, unsigned int numParticles);
#endif

#endif /* __cplusplus */
#endif /* FCDEM_I3D_H */
