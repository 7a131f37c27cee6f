/*
 * fcdem_particledem.h -- the C++ particledem interface of FullC0ntact
 * (cuda_addon/particledem.cuh:11-26: calcHash / sortParticles /
 * reorderDataAndFindCellStart / evalForces on HashGrid + ParticleWorld
 * objects, and the unified-memory set of cuda_addon/particledem_um.cuh:11-27)
 * over libfcdem's C-ABI.  Header only.
 *
 * HashGrid and ParticleWorld keep the field names of
 * inshape3dcore/grid/uniformgrid.h:495-589 (HashGrid<T,memory>,
 * ParticleWorld<T,memory>); the simulation parameters are the 104-byte
 * SimParams of the particleSystem interface instead of
 * SimulationParameters<T>.  All pointers are device pointers, positions and
 * velocities 4 floats per particle, force_ 3 floats per particle.
 */
#ifndef FCDEM_PARTICLEDEM_H
#define FCDEM_PARTICLEDEM_H

#include "fcdem.h"

#ifdef __cplusplus
namespace fcdem {

struct HashGrid {
  unsigned int size_ = 0;
  unsigned int numCells_ = 0;
  unsigned int *hashEntries_ = nullptr;
  unsigned int *particleIndices_ = nullptr;
  unsigned int *cellStart_ = nullptr;
  unsigned int *cellEnd_ = nullptr;
  unsigned int gridx_ = 0, gridy_ = 0, gridz_ = 0;
};

struct ParticleWorld {
  SimParams params_{};
  float *pos_ = nullptr;
  float *vel_ = nullptr;
  float *sortedPos_ = nullptr;
  float *sortedVel_ = nullptr;
  float *force_ = nullptr;  /* particledem_um's extra output */
  int size_ = 0;
  bool radiusFromW_ = false;
};

/* particledem.cu:122-160 */
inline void calcHash(HashGrid &hg, ParticleWorld &pw) {
  setParameters(&pw.params_);
  fcdemSetRadiusMode(pw.radiusFromW_ ? 1 : 0);
  ::calcHash(hg.hashEntries_, hg.particleIndices_, pw.pos_, pw.size_);
}

/* particledem.cu:222-231 (thrust::sort_by_key on the grid's arrays) */
inline void sortParticles(HashGrid &hg) {
  ::sortParticles(hg.hashEntries_, hg.particleIndices_, hg.size_);
}

/* particledem.cu:163-234: both cell tables reset, then ranges and gathers */
inline void reorderDataAndFindCellStart(HashGrid &hg, ParticleWorld &pw) {
  fcdemUM_reorderDataAndFindCellStart(hg.cellStart_, hg.cellEnd_, pw.sortedPos_,
                                      pw.sortedVel_, hg.hashEntries_, hg.particleIndices_,
                                      pw.pos_, pw.vel_, (uint)pw.size_, hg.numCells_);
}

/* particledem.cu:236-409 / particledem_um.cu:457-602: pair forces without
 * the collider sphere; vel_ receives v + F, force_ (when set) receives F. */
inline void evalForces(HashGrid &hg, ParticleWorld &pw) {
  setParameters(&pw.params_);
  fcdemSetRadiusMode(pw.radiusFromW_ ? 1 : 0);
  if (pw.force_) {
    fcdemUM_evalForces(pw.vel_, pw.force_, pw.sortedPos_, pw.sortedVel_,
                       hg.particleIndices_, hg.cellStart_, hg.cellEnd_, (uint)pw.size_,
                       hg.numCells_);
  } else {
    /* the particleSystem collide adds the collider sphere: keep it out by
     * parking the collider at radius 0 */
    SimParams p = pw.params_;
    p.colliderRadius = 0.0f;
    p.colliderPos[0] = p.colliderPos[1] = p.colliderPos[2] = 3.0e38f;
    setParameters(&p);
    collide(pw.vel_, pw.sortedPos_, pw.sortedVel_, hg.particleIndices_, hg.cellStart_,
            hg.cellEnd_, (uint)pw.size_, hg.numCells_);
    setParameters(&pw.params_);
  }
}

/* particledem_um.cu:720-734: integrate with the distance-map boundary */
inline void integrateSystem(ParticleWorld &pw, float deltaTime, const fcdemDistanceMap *map) {
  setParameters(&pw.params_);
  fcdemSetRadiusMode(pw.radiusFromW_ ? 1 : 0);
  fcdemUM_integrateSystem(pw.pos_, pw.vel_, deltaTime, (uint)pw.size_, map);
}

}  // namespace fcdem
#endif

#endif
