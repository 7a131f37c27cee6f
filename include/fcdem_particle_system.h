/*
 * fcdem_particle_system.h -- headless C++ counterpart of FullC0ntact's
 * ParticleSystem (cuda_addon/particleSystem.h:22-136,
 * cuda_addon/particleSystem.cpp:30-509) on top of libfcdem's C-ABI.
 *
 * Same constructor defaults, setters/getters, host mirrors m_hPos/m_hVel and
 * update() order (integrate, hash, sort, reorder, collide).  OpenGL buffers
 * are replaced by plain device buffers: constructing with bUseOpenGL = true
 * records FCDEM_ERR_UNSUPPORTED and continues headless.
 *
 * A C wrapper (fcdemPS_*) follows for FFI callers.
 */
#ifndef FCDEM_PARTICLE_SYSTEM_H
#define FCDEM_PARTICLE_SYSTEM_H

#include "fcdem.h"

#ifdef __cplusplus
namespace fcdem {

class ParticleSystem {
 public:
  enum ParticleConfig { CONFIG_RANDOM, CONFIG_GRID, _NUM_CONFIGS };
  enum ParticleArray { POSITION, VELOCITY };

  /* particleSystem.cpp:30-72; gridSize is {x, y, z}. */
  ParticleSystem(uint numParticles, const uint gridSize[3], bool bUseOpenGL);
  ~ParticleSystem();

  /* particleSystem.cpp:222-284.  With setFusedUpdate(true) (the default) the
   * five stages run as the fused sequence of fcdemUpdate, which leaves the
   * same state. */
  void update(float deltaTime);
  /* `steps` updates in one fused call. */
  void updateSteps(float deltaTime, uint steps);
  void reset(ParticleConfig config);
  void setParticles(const float *positions, const float *velocities);
  void setVelocity(const float *velocities);

  float *getArray(ParticleArray array);
  void setArray(ParticleArray array, const float *data, int start, int count);

  int getNumParticles() const { return (int)m_numParticles; }
  float *getDevicePos() const { return m_dPos; }
  float *getDeviceVel() const { return m_dVel; }

  /* maximum particles per cell (particleSystem.cpp:286-301), returned
   * instead of printed */
  uint dumpGrid();
  void transferArrays(uint start, uint count);

  void setIterations(int i) { m_solverIterations = i; }
  void setDamping(float x) { m_params.globalDamping = x; }
  void setGravity(float x) {
    m_params.gravity[0] = 0.0f; m_params.gravity[1] = 0.0f; m_params.gravity[2] = x;
  }
  void setCollideSpring(float x) { m_params.spring = x; }
  void setCollideDamping(float x) { m_params.damping = x; }
  void setCollideShear(float x) { m_params.shear = x; }
  void setCollideAttraction(float x) { m_params.attraction = x; }
  void setColliderPos(const float x[3]) {
    for (int k = 0; k < 3; ++k) m_params.colliderPos[k] = x[k];
  }
  float getParticleRadius() const { return m_params.particleRadius; }
  float getColliderRadius() const { return m_params.colliderRadius; }
  SimParams &params() { return m_params; }

  void setFusedUpdate(bool fused) { m_fused = fused; }
  /* polydisperse mode: radius of particle i in pos[i].w */
  void setRadiusFromW(bool on) { m_radiusFromW = on; }

  /* particleSystem.cpp:617-647 */
  void addSphere(int start, const float *pos, const float *vel, int r, float spacing);

  float *m_hPos;  /* host mirrors, 4 floats per particle */
  float *m_hVel;

 protected:
  void _initialize(int numParticles);
  void _finalize();
  void initGrid(const uint size[3], float spacing, float jitter, uint numParticles);
  float frand();

  bool m_bInitialized, m_bUseOpenGL, m_fused, m_radiusFromW;
  uint m_numParticles;
  uint *m_hCellStart, *m_hCellEnd;
  float *m_dPos, *m_dVel, *m_dSortedPos, *m_dSortedVel;
  uint *m_dGridParticleHash, *m_dGridParticleIndex, *m_dCellStart, *m_dCellEnd;
  SimParams m_params;
  uint m_gridSize[3];
  uint m_numGridCells;
  int m_solverIterations;
  unsigned long long m_rng;
};

}  // namespace fcdem
extern "C" {
#endif

/* C wrapper of fcdem::ParticleSystem. */
typedef struct fcdemParticleSystem fcdemParticleSystem;
fcdemParticleSystem *fcdemPS_create(uint numParticles, uint gx, uint gy, uint gz);
void fcdemPS_destroy(fcdemParticleSystem *ps);
SimParams *fcdemPS_params(fcdemParticleSystem *ps);
void fcdemPS_update(fcdemParticleSystem *ps, float deltaTime);
void fcdemPS_updateSteps(fcdemParticleSystem *ps, float deltaTime, uint steps);
void fcdemPS_reset(fcdemParticleSystem *ps, int config);
void fcdemPS_setArray(fcdemParticleSystem *ps, int array, const float *data, int start, int count);
const float *fcdemPS_getArray(fcdemParticleSystem *ps, int array);
uint fcdemPS_dumpGrid(fcdemParticleSystem *ps);
void fcdemPS_setFusedUpdate(fcdemParticleSystem *ps, int fused);
void fcdemPS_setRadiusFromW(fcdemParticleSystem *ps, int on);
float *fcdemPS_devicePos(fcdemParticleSystem *ps);
float *fcdemPS_deviceVel(fcdemParticleSystem *ps);

#ifdef __cplusplus
}
#endif

#endif
