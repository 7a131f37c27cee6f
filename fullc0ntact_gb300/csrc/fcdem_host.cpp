// fcdem_host.cpp -- host side above the C-ABI: the headless ParticleSystem
// (cuda_addon/particleSystem.cpp) and the VTK particle writer.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/fcdem.h"
#include "../../include/fcdem_particle_system.h"
#include "fcdem_rng.h"

using fcdem_rng::uniformF;

namespace {

// The legacy ASCII VTK particle file of CVtkWriter::WriteGPUParticleFile
// (inshape3dcore/postprocessing/vtkwriter.cpp:3399-3452): header, the points,
// a "radius" scalar (radiusOf(i)), a "myid" scalar, and -- when vel4 is not
// NULL -- a "velocity" vector.
template <class RadiusOf>
int writeParticleVtk(const char *path, const char *generator, const float *pos4,
                     const float *vel4, uint n, RadiusOf radiusOf) {
  if (!path || (n && !pos4)) return FCDEM_ERR_INVALID_VALUE;
  FILE *f = std::fopen(path, "w");
  if (!f) return FCDEM_ERR_INVALID_VALUE;
  std::fprintf(f, "# vtk DataFile Version 2.0\n");
  std::fprintf(f, "Generated by %s\n", generator);
  std::fprintf(f, "ASCII\n");
  std::fprintf(f, "DATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %u double\n", n);
  for (uint i = 0; i < n; ++i)
    std::fprintf(f, "%f %f %f \n", pos4[4 * (size_t)i], pos4[4 * (size_t)i + 1],
                 pos4[4 * (size_t)i + 2]);
  std::fprintf(f, "POINT_DATA %u\n", n);
  std::fprintf(f, "SCALARS radius double 1\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (uint i = 0; i < n; ++i) std::fprintf(f, "%f \n", radiusOf(i));
  std::fprintf(f, "SCALARS myid double 1\n");
  std::fprintf(f, "LOOKUP_TABLE default\n");
  for (uint i = 0; i < n; ++i) std::fprintf(f, "%f \n", (float)i);
  if (vel4) {
    std::fprintf(f, "VECTORS velocity double\n");
    for (uint i = 0; i < n; ++i)
      std::fprintf(f, "%f %f %f \n", vel4[4 * (size_t)i], vel4[4 * (size_t)i + 1],
                   vel4[4 * (size_t)i + 2]);
  }
  int bad = std::ferror(f);
  std::fclose(f);
  return bad ? FCDEM_ERR_INVALID_VALUE : FCDEM_SUCCESS;
}

}  // namespace

extern "C" int fcdemWriteVtkParticles(const char *path, const float *pos4, const float *vel4,
                                      uint n, float radius, int radiusFromW) {
  return writeParticleVtk(path, "fcdem-gb300", pos4, vel4, n, [&](uint i) {
    return radiusFromW ? pos4[4 * (size_t)i + 3] : radius;
  });
}

extern "C" int fcdemWriteGPUParticleFile(const float *pos4, uint n, const char *path) {
  // the reference's own bytes: its generator line and a radius of 1/64 for
  // every particle, no velocity
  return writeParticleVtk(path, "InShape 2.x", pos4, nullptr, n,
                          [](uint) { return 1.0f / 64.0f; });
}

// ---------------------------------------------------------------------------
namespace fcdem {

ParticleSystem::ParticleSystem(uint numParticles, const uint gridSize[3], bool bUseOpenGL)
    : m_hPos(nullptr), m_hVel(nullptr), m_bInitialized(false), m_bUseOpenGL(false),
      m_fused(true), m_radiusFromW(false), m_numParticles(numParticles),
      m_hCellStart(nullptr), m_hCellEnd(nullptr), m_dPos(nullptr), m_dVel(nullptr),
      m_dSortedPos(nullptr), m_dSortedVel(nullptr), m_dGridParticleHash(nullptr),
      m_dGridParticleIndex(nullptr), m_dCellStart(nullptr), m_dCellEnd(nullptr),
      m_solverIterations(1), m_rng(1973) {
  if (bUseOpenGL) registerGLBufferObject(0, nullptr);  // records UNSUPPORTED
  for (int k = 0; k < 3; ++k) m_gridSize[k] = gridSize[k];
  m_numGridCells = m_gridSize[0] * m_gridSize[1] * m_gridSize[2];
  std::memset(&m_params, 0, sizeof(m_params));
  // particleSystem.cpp:36-70
  for (int k = 0; k < 3; ++k) m_params.gridSize[k] = m_gridSize[k];
  m_params.numCells = m_numGridCells;
  m_params.numBodies = m_numParticles;
  m_params.particleRadius = 1.0f / 16.0f;
  m_params.colliderPos[0] = -1.2f;
  m_params.colliderPos[1] = -0.8f;
  m_params.colliderPos[2] = 0.8f;
  m_params.colliderRadius = 0.2f;
  for (int k = 0; k < 3; ++k) m_params.worldOrigin[k] = -1.0f;
  float cellSize = m_params.particleRadius * 2.0f;
  for (int k = 0; k < 3; ++k) m_params.cellSize[k] = cellSize;
  m_params.spring = 0.5f;
  m_params.damping = 0.02f;
  m_params.shear = 0.1f;
  m_params.attraction = 0.0f;
  m_params.boundaryDamping = -0.5f;
  m_params.gravity[0] = 0.0f;
  m_params.gravity[1] = 0.0f;
  m_params.gravity[2] = -0.0003f;
  m_params.globalDamping = 1.0f;
  _initialize((int)numParticles);
}

ParticleSystem::~ParticleSystem() {
  _finalize();
  m_numParticles = 0;
}

void ParticleSystem::_initialize(int numParticles) {
  m_numParticles = (uint)numParticles;
  size_t n4 = (size_t)m_numParticles * 4;
  m_hPos = new float[n4]();
  m_hVel = new float[n4]();
  m_hCellStart = new uint[m_numGridCells]();
  m_hCellEnd = new uint[m_numGridCells]();
  // byte counts as int, as particleSystem.cpp:117-190 passes them
  const int memSize = (int)(sizeof(float) * n4);
  allocateArray((void **)&m_dPos, memSize);
  allocateArray((void **)&m_dVel, memSize);
  allocateArray((void **)&m_dSortedPos, memSize);
  allocateArray((void **)&m_dSortedVel, memSize);
  allocateArray((void **)&m_dGridParticleHash, (int)(m_numParticles * sizeof(uint)));
  allocateArray((void **)&m_dGridParticleIndex, (int)(m_numParticles * sizeof(uint)));
  allocateArray((void **)&m_dCellStart, (int)(m_numGridCells * sizeof(uint)));
  allocateArray((void **)&m_dCellEnd, (int)(m_numGridCells * sizeof(uint)));
  setParameters(&m_params);
  m_bInitialized = true;
}

void ParticleSystem::_finalize() {
  if (!m_bInitialized) return;
  delete[] m_hPos;
  delete[] m_hVel;
  delete[] m_hCellStart;
  delete[] m_hCellEnd;
  freeArray(m_dPos);
  freeArray(m_dVel);
  freeArray(m_dSortedPos);
  freeArray(m_dSortedVel);
  freeArray(m_dGridParticleHash);
  freeArray(m_dGridParticleIndex);
  freeArray(m_dCellStart);
  freeArray(m_dCellEnd);
  m_bInitialized = false;
}

void ParticleSystem::update(float deltaTime) { updateSteps(deltaTime, 1); }

void ParticleSystem::updateSteps(float deltaTime, uint steps) {
  if (!m_bInitialized || steps == 0) return;
  setParameters(&m_params);
  fcdemSetRadiusMode(m_radiusFromW ? 1 : 0);
  if (m_fused) {
    fcdemUpdate(m_dPos, m_dVel, m_dSortedPos, m_dSortedVel, m_dGridParticleHash,
                m_dGridParticleIndex, m_dCellStart, m_dCellEnd, deltaTime,
                m_numParticles, m_numGridCells, steps);
    return;
  }
  for (uint s = 0; s < steps; ++s) {  // particleSystem.cpp:236-281
    integrateSystem(m_dPos, m_dVel, deltaTime, m_numParticles);
    calcHash(m_dGridParticleHash, m_dGridParticleIndex, m_dPos, (int)m_numParticles);
    sortParticles(m_dGridParticleHash, m_dGridParticleIndex, m_numParticles);
    reorderDataAndFindCellStart(m_dCellStart, m_dCellEnd, m_dSortedPos, m_dSortedVel,
                                m_dGridParticleHash, m_dGridParticleIndex, m_dPos,
                                m_dVel, m_numParticles, m_numGridCells);
    collide(m_dVel, m_dSortedPos, m_dSortedVel, m_dGridParticleIndex, m_dCellStart,
            m_dCellEnd, m_numParticles, m_numGridCells);
  }
}

uint ParticleSystem::dumpGrid() {
  copyArrayFromDevice(m_hCellStart, m_dCellStart, nullptr, (int)(sizeof(uint) * m_numGridCells));
  copyArrayFromDevice(m_hCellEnd, m_dCellEnd, nullptr, (int)(sizeof(uint) * m_numGridCells));
  uint maxCellSize = 0;
  for (uint i = 0; i < m_numGridCells; i++)
    if (m_hCellStart[i] != 0xffffffffu)
      maxCellSize = std::max(maxCellSize, m_hCellEnd[i] - m_hCellStart[i]);
  return maxCellSize;
}

void ParticleSystem::transferArrays(uint start, uint count) {
  (void)start;
  copyArrayFromDevice(m_hPos, m_dPos, nullptr, (int)(sizeof(float) * 4 * count));
  copyArrayFromDevice(m_hVel, m_dVel, nullptr, (int)(sizeof(float) * 4 * count));
}

float *ParticleSystem::getArray(ParticleArray array) {
  float *h = array == VELOCITY ? m_hVel : m_hPos;
  float *d = array == VELOCITY ? m_dVel : m_dPos;
  copyArrayFromDevice(h, d, nullptr, (int)(m_numParticles * 4 * sizeof(float)));
  return h;
}

void ParticleSystem::setArray(ParticleArray array, const float *data, int start, int count) {
  float *d = array == VELOCITY ? m_dVel : m_dPos;
  copyArrayToDevice(d, data, start * 4 * (int)sizeof(float), count * 4 * (int)sizeof(float));
}

float ParticleSystem::frand() { return uniformF(m_rng); }

void ParticleSystem::initGrid(const uint size[3], float spacing, float jitter,
                              uint numParticles) {  // particleSystem.cpp:380-402
  for (uint z = 0; z < size[2]; z++)
    for (uint y = 0; y < size[1]; y++)
      for (uint x = 0; x < size[0]; x++) {
        uint i = (z * size[1] * size[0]) + (y * size[0]) + x;
        if (i < numParticles) {
          m_hPos[i * 4] = (spacing * x) + m_params.particleRadius - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[i * 4 + 1] = (spacing * y) + m_params.particleRadius - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[i * 4 + 2] = (spacing * z) + m_params.particleRadius - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[i * 4 + 3] = 1.0f;
          m_hVel[i * 4] = m_hVel[i * 4 + 1] = m_hVel[i * 4 + 2] = m_hVel[i * 4 + 3] = 0.0f;
        }
      }
}

void ParticleSystem::reset(ParticleConfig config) {  // particleSystem.cpp:404-444
  m_rng = 1973;
  if (config == CONFIG_GRID) {
    float jitter = m_params.particleRadius * 0.01f;
    uint s = (uint)std::ceil(std::pow((float)m_numParticles, 1.0f / 3.0f));
    uint gs[3] = {s, s, s};
    initGrid(gs, m_params.particleRadius * 2.0f, jitter, m_numParticles);
  } else {
    size_t p = 0, v = 0;
    for (uint i = 0; i < m_numParticles; i++) {
      float pt[3] = {frand(), frand(), frand()};
      m_hPos[p++] = 2 * (pt[0] - 0.5f);
      m_hPos[p++] = 2 * (pt[1] - 0.5f);
      m_hPos[p++] = 2 * (pt[2] - 0.5f);
      m_hPos[p++] = 1.0f;
      m_hVel[v++] = 0.0f; m_hVel[v++] = 0.0f; m_hVel[v++] = 0.0f; m_hVel[v++] = 0.0f;
    }
  }
  setArray(POSITION, m_hPos, 0, (int)m_numParticles);
  setArray(VELOCITY, m_hVel, 0, (int)m_numParticles);
}

void ParticleSystem::setParticles(const float *positions, const float *velocities) {
  for (uint i = 0; i < m_numParticles; i++) {
    for (int k = 0; k < 3; ++k) {
      m_hPos[i * 4 + k] = positions[i * 4 + k];
      m_hVel[i * 4 + k] = velocities[i * 4 + k];
    }
    m_hPos[i * 4 + 3] = m_radiusFromW ? positions[i * 4 + 3] : 1.0f;
    m_hVel[i * 4 + 3] = 0.0f;
  }
  setArray(POSITION, m_hPos, 0, (int)m_numParticles);
  setArray(VELOCITY, m_hVel, 0, (int)m_numParticles);
}

void ParticleSystem::setVelocity(const float *velocities) {
  for (uint i = 0; i < m_numParticles; i++) {
    for (int k = 0; k < 3; ++k) m_hVel[i * 4 + k] = velocities[i * 4 + k];
    m_hVel[i * 4 + 3] = 0.0f;
  }
  setArray(VELOCITY, m_hVel, 0, (int)m_numParticles);
}

void ParticleSystem::addSphere(int start, const float *pos, const float *vel, int r,
                               float spacing) {  // particleSystem.cpp:617-647
  uint index = (uint)start;
  for (int z = -r; z <= r; z++)
    for (int y = -r; y <= r; y++)
      for (int x = -r; x <= r; x++) {
        float dx = x * spacing, dy = y * spacing, dz = z * spacing;
        float l = std::sqrt(dx * dx + dy * dy + dz * dz);
        float jitter = m_params.particleRadius * 0.01f;
        if ((l <= m_params.particleRadius * 2.0f * r) && (index < m_numParticles)) {
          m_hPos[index * 4] = pos[0] + dx + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[index * 4 + 1] = pos[1] + dy + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[index * 4 + 2] = pos[2] + dz + (frand() * 2.0f - 1.0f) * jitter;
          m_hPos[index * 4 + 3] = pos[3];
          for (int k = 0; k < 4; ++k) m_hVel[index * 4 + k] = vel[k];
          index++;
        }
      }
  setArray(POSITION, m_hPos + 4 * (size_t)start, start, (int)(index - (uint)start));
  setArray(VELOCITY, m_hVel + 4 * (size_t)start, start, (int)(index - (uint)start));
}

}  // namespace fcdem

// ---------------------------------------------------------------------------
struct fcdemParticleSystem {
  fcdem::ParticleSystem ps;
  fcdemParticleSystem(uint n, const uint g[3]) : ps(n, g, false) {}
};

extern "C" {

fcdemParticleSystem *fcdemPS_create(uint numParticles, uint gx, uint gy, uint gz) {
  uint g[3] = {gx, gy, gz};
  return new fcdemParticleSystem(numParticles, g);
}
void fcdemPS_destroy(fcdemParticleSystem *ps) { delete ps; }
SimParams *fcdemPS_params(fcdemParticleSystem *ps) { return &ps->ps.params(); }
void fcdemPS_update(fcdemParticleSystem *ps, float dt) { ps->ps.update(dt); }
void fcdemPS_updateSteps(fcdemParticleSystem *ps, float dt, uint steps) {
  ps->ps.updateSteps(dt, steps);
}
void fcdemPS_reset(fcdemParticleSystem *ps, int config) {
  ps->ps.reset(config == 1 ? fcdem::ParticleSystem::CONFIG_GRID
                           : fcdem::ParticleSystem::CONFIG_RANDOM);
}
void fcdemPS_setArray(fcdemParticleSystem *ps, int array, const float *data, int start,
                      int count) {
  ps->ps.setArray(array == 1 ? fcdem::ParticleSystem::VELOCITY
                             : fcdem::ParticleSystem::POSITION,
                  data, start, count);
}
const float *fcdemPS_getArray(fcdemParticleSystem *ps, int array) {
  return ps->ps.getArray(array == 1 ? fcdem::ParticleSystem::VELOCITY
                                    : fcdem::ParticleSystem::POSITION);
}
uint fcdemPS_dumpGrid(fcdemParticleSystem *ps) { return ps->ps.dumpGrid(); }
void fcdemPS_setFusedUpdate(fcdemParticleSystem *ps, int fused) {
  ps->ps.setFusedUpdate(fused != 0);
}
void fcdemPS_setRadiusFromW(fcdemParticleSystem *ps, int on) {
  ps->ps.setRadiusFromW(on != 0);
}
float *fcdemPS_devicePos(fcdemParticleSystem *ps) { return ps->ps.getDevicePos(); }
float *fcdemPS_deviceVel(fcdemParticleSystem *ps) { return ps->ps.getDeviceVel(); }

}  // extern "C"
