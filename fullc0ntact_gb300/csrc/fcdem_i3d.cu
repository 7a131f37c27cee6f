// fcdem_i3d.cu -- the particledem C++ interface (cuda_addon/particledem.cuh:
// 11-26, implemented in cuda_addon/particledem.cu:26-460) on the i3d
// container types, over the kernels of the particleSystem stages.
//
// The reference keeps a device copy of its HashGrid and ParticleWorld made
// at cuda_init and launches on those; here the host objects passed to each
// call carry the device arrays (cuda_init stores their addresses in them, as
// the reference's deepCopy does), and the contact parameters are the copy
// taken at cuda_init.  integrateSystem (C++ linkage) is defined in
// fcdem_i3d_integrate.cpp: this file sees fcdem.h's extern "C" declaration
// of the same name.
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "fcdem_dem.cuh"
#define FCDEM_I3D_NO_INTEGRATE_DECL
#include "../../include/fcdem_i3d.h"

namespace fcdem {
namespace {

// What cuda_init captured: the parameter block of the particledem step and
// the device copy of the SimulationParameters it hands back.
struct I3dWorld {
  bool ready = false;
  SimParams p{};
  i3d::SimulationParameters<float> *devParams = nullptr;
};
I3dWorld g_i3d;
std::mutex g_i3dMutex;

// The parameter block for a call: the contact parameters taken at cuda_init
// (no collider sphere: evalForces has none), the grid of hg.
bool paramsFor(const i3d::HashGrid<float, i3d::cpu> &hg, KParams &kp) {
  std::lock_guard<std::mutex> lock(g_i3dMutex);
  if (!g_i3d.ready) { setError(FCDEM_ERR_NO_PARAMS); return false; }
  kp.p = g_i3d.p;
  kp.p.gridSize[0] = hg.gridx_;
  kp.p.gridSize[1] = hg.gridy_;
  kp.p.gridSize[2] = hg.gridz_;
  kp.p.numCells = hg.numCells_;
  kp.p.worldOrigin[0] = hg.origin_.x;
  kp.p.worldOrigin[1] = hg.origin_.y;
  kp.p.worldOrigin[2] = hg.origin_.z;
  kp.p.cellSize[0] = hg.cellSize_.x;
  kp.p.cellSize[1] = hg.cellSize_.y;
  kp.p.cellSize[2] = hg.cellSize_.z;
  kp.p.maxParticlesPerCell = 0u;
  kp.radiusFromW = 0;
  for (int k = 0; k < 3; ++k) {
    const unsigned g = kp.p.gridSize[k];
    if (g == 0 || (g & (g - 1)) != 0) { setError(FCDEM_ERR_INVALID_VALUE); return false; }
  }
  if ((unsigned long long)hg.gridx_ * hg.gridy_ * hg.gridz_ > hg.numCells_) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return false;
  }
  return true;
}

template <class T>
bool deviceAlloc(T *&p, size_t count) {
  p = nullptr;
  if (cudaMalloc((void **)&p, count * sizeof(T) + (count == 0)) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    setError(FCDEM_ERR_ALLOC);
    return false;
  }
  return true;
}

}  // namespace

// particledem.cu:412-460: integrate in [-1, 1]^3 with the parameters taken
// at cuda_init (called by the C++-linkage integrateSystem).
void i3dIntegrate(float *pos, float *vel, float dt, unsigned n) {
  KParams kp;
  {
    std::lock_guard<std::mutex> lock(g_i3dMutex);
    if (!g_i3d.ready) { setError(FCDEM_ERR_NO_PARAMS); return; }
    kp.p = g_i3d.p;
    kp.radiusFromW = 0;
  }
  if (n == 0) return;
  if (!pos || !vel) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  launchIntegrate((float4 *)pos, (float4 *)vel, dt, n, kp);
}

}  // namespace fcdem

using namespace fcdem;

// particledem.cu:86-120 (with initGrid, :47-75).
void cuda_init(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw,
               i3d::SimulationParameters<float> *&params) {
  if (!pw.params_ || pw.size_ < 0) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  const i3d::SimulationParameters<float> &sp = *pw.params_;
  const float r = sp.particleRadius_;
  hg.cellSize_.x = hg.cellSize_.y = hg.cellSize_.z = 2.0f * r;
  hg.origin_ = sp.origin_;
  hg.gridx_ = sp.gridx_;
  hg.gridy_ = sp.gridy_;
  hg.gridz_ = sp.gridz_;
  hg.numCells_ = hg.gridx_ * hg.gridy_ * hg.gridz_;
  const size_t n = (size_t)pw.size_;
  if (!deviceAlloc(hg.hashEntries_, hg.size_) || !deviceAlloc(hg.particleIndices_, hg.size_) ||
      !deviceAlloc(hg.cellStart_, hg.numCells_) || !deviceAlloc(hg.cellEnd_, hg.numCells_) ||
      !deviceAlloc(pw.pos_, 4 * n) || !deviceAlloc(pw.vel_, 4 * n) ||
      !deviceAlloc(pw.sortedPos_, 4 * n) || !deviceAlloc(pw.sortedVel_, 4 * n))
    return;
  i3d::SimulationParameters<float> *dev = nullptr;
  if (!deviceAlloc(dev, 1) || !cudaOk(cudaMemcpy(dev, pw.params_, sizeof(*dev),
                                                 cudaMemcpyHostToDevice)))
    return;
  params = dev;
  {
    std::lock_guard<std::mutex> lock(g_i3dMutex);
    SimParams p{};
    p.gravity[0] = sp.gravity_.x;
    p.gravity[1] = sp.gravity_.y;
    p.gravity[2] = sp.gravity_.z;
    p.globalDamping = sp.globalDamping_;
    p.particleRadius = r;
    p.spring = sp.spring_;
    p.damping = sp.damping_;
    p.shear = sp.shear_;
    p.attraction = sp.attraction_;
    p.boundaryDamping = sp.boundaryDamping_;
    g_i3d.p = p;
    g_i3d.devParams = dev;
    g_i3d.ready = true;
  }
  // initGrid: a jittered cubic lattice of spacing 2r from (-1, -1, -1),
  // jitter 0.01 r from srand(1973) / rand(), velocities zero.
  const unsigned s = (unsigned)std::ceil(std::pow((float)pw.size_, 1.0f / 3.0f));
  const float spacing = 2.0f * r, jitter = r * 0.01f;
  std::vector<float> pos(4 * n, 0.0f), vel(4 * n, 0.0f);
  std::srand(1973);
  auto frand = []() { return std::rand() / (float)RAND_MAX; };
  for (unsigned z = 0; z < s; ++z)
    for (unsigned y = 0; y < s; ++y)
      for (unsigned x = 0; x < s; ++x) {
        const size_t i = ((size_t)z * s + y) * s + x;
        if (i >= n) continue;
        pos[4 * i] = (spacing * x) + r - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
        pos[4 * i + 1] = (spacing * y) + r - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
        pos[4 * i + 2] = (spacing * z) + r - 1.0f + (frand() * 2.0f - 1.0f) * jitter;
        pos[4 * i + 3] = 1.0f;
      }
  if (n) {
    cudaOk(cudaMemcpy(pw.pos_, pos.data(), 16 * n, cudaMemcpyHostToDevice));
    cudaOk(cudaMemcpy(pw.vel_, vel.data(), 16 * n, cudaMemcpyHostToDevice));
  }
}

// particledem.cu:26-30
void cuda_clean() {
  std::lock_guard<std::mutex> lock(g_i3dMutex);
  if (g_i3d.devParams) cudaFree(g_i3d.devParams);
  g_i3d.devParams = nullptr;
  g_i3d.ready = false;
}

// particledem.cu:154-162 (calcHashD, :122-146): hashes of pw.size_ particles.
void calcHash(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw) {
  KParams kp;
  if (!paramsFor(hg, kp)) return;
  if (pw.size_ <= 0) return;
  if (!hg.hashEntries_ || !hg.particleIndices_ || !pw.pos_ || (unsigned)pw.size_ > hg.size_) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  launchCalcHash(hg.hashEntries_, hg.particleIndices_, (const float4 *)pw.pos_,
                 (unsigned)pw.size_, kp);
}

// particledem.cu:81-84 (HashGrid<gpu>::sortParticles, uniformgrid.cuh:95-100):
// stable sort of hg.size_ (hash, index) pairs.
void sortParticles(i3d::HashGrid<float, i3d::cpu> &hg) {
  if (hg.size_ < 2) return;
  if (!hg.hashEntries_ || !hg.particleIndices_) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  radixSortPairs(ctx(), hg.hashEntries_, hg.particleIndices_, hg.size_, keyBits(hg.numCells_));
}

// particledem.cu:223-234 (reorderDataAndFindCellStartD, :164-221): cellStart
// and cellEnd of every cell set to 0xffffffff first.
void reorderDataAndFindCellStart(i3d::HashGrid<float, i3d::cpu> &hg,
                                 i3d::ParticleWorld<float, i3d::cpu> &pw) {
  if (!hg.cellStart_ || !hg.cellEnd_ ||
      (pw.size_ > 0 && (!hg.hashEntries_ || !hg.particleIndices_ || !pw.pos_ || !pw.vel_ ||
                        !pw.sortedPos_ || !pw.sortedVel_))) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  Context &c = ctx();
  fillU32(c, hg.cellStart_, hg.numCells_, 0xffffffffu);
  fillU32(c, hg.cellEnd_, hg.numCells_, 0xffffffffu);
  if (pw.size_ <= 0) return;
  launchReorder(hg.cellStart_, hg.cellEnd_, (float4 *)pw.sortedPos_, (float4 *)pw.sortedVel_,
                hg.hashEntries_, hg.particleIndices_, (const float4 *)pw.pos_,
                (const float4 *)pw.vel_, (unsigned)pw.size_, hg.numCells_);
}

// particledem.cu:399-408 (evalForces_launcher, :349-397): the pair forces
// over the 27 neighbour cells, no collider, pw.vel_[index[i]] = v + F.
void evalForces(i3d::HashGrid<float, i3d::cpu> &hg, i3d::ParticleWorld<float, i3d::cpu> &pw) {
  KParams kp;
  if (!paramsFor(hg, kp)) return;
  if (pw.size_ <= 0) return;
  if (!pw.vel_ || !pw.sortedPos_ || !pw.sortedVel_ || !hg.particleIndices_ || !hg.cellStart_ ||
      !hg.cellEnd_) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  CellRanges cells;
  cells.start = hg.cellStart_;
  cells.end = hg.cellEnd_;
  launchCollide(0, false, (float4 *)pw.vel_, (const float4 *)pw.sortedPos_,
                (const float4 *)pw.sortedVel_, hg.particleIndices_, cells, (unsigned)pw.size_,
                kp, CollideOut());
}
