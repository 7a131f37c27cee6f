// fcdem_scenes.cpp -- the seeded scene generators of the C-ABI
// (fcdemSceneLattice, fcdemScenePack, fcdemScenePackRadii): host code only,
// compiled into libfcdem.so and, from this same file, into the small
// generator library the benchmark's reference arm uses to build its workload
// without the GPU library.  Compiled with -ffp-contract=off in both builds,
// so that a seed gives the same scene in both.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/fcdem.h"

#include "fcdem_rng.h"

using fcdem_rng::u64;
using fcdem_rng::uniformD;
using fcdem_rng::uniformF;

extern "C" void fcdemSceneLattice(float *pos4, float *vel4, uint n, float radius,
                                  float spacing, float jitter, float velRange,
                                  unsigned long long seed) {
  u64 s = seed;
  uint side = (uint)std::ceil(std::pow((double)n, 1.0 / 3.0));
  while ((uint64_t)side * side * side < n) ++side;
  uint i = 0;
  for (uint z = 0; z < side && i < n; ++z)
    for (uint y = 0; y < side && i < n; ++y)
      for (uint x = 0; x < side && i < n; ++x, ++i) {
        float c[3] = {(float)x, (float)y, (float)z};
        for (int k = 0; k < 3; ++k)
          pos4[4 * (size_t)i + k] =
              (spacing * c[k]) + radius - 1.0f + (uniformF(s) * 2.0f - 1.0f) * jitter;
        pos4[4 * (size_t)i + 3] = 1.0f;
        for (int k = 0; k < 3; ++k)
          vel4[4 * (size_t)i + k] = (uniformF(s) * 2.0f - 1.0f) * velRange;
        vel4[4 * (size_t)i + 3] = 0.0f;
      }
}

extern "C" uint fcdemScenePack(float *pos4, float *vel4, uint n, const float boxMin[3],
                               const float boxMax[3], float rMedian, float sigma,
                               float rMax, float velRange, unsigned long long seed,
                               uint maxAttempts) {
  u64 s = seed;
  std::vector<float> radii(n);
  for (uint i = 0; i < n; ++i) {
    // Box-Muller normal, then lognormal around the median.
    double u1 = uniformD(s), u2 = uniformD(s);
    if (u1 < 1e-300) u1 = 1e-300;
    double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    double r = (double)rMedian * std::exp((double)sigma * z);
    radii[i] = (float)std::min(r, (double)rMax);
  }
  return fcdemScenePackRadii(pos4, vel4, n, radii.data(), boxMin, boxMax, velRange, s,
                             maxAttempts);
}

extern "C" uint fcdemScenePackRadii(float *pos4, float *vel4, uint n, const float *radiiIn,
                                    const float boxMin[3], const float boxMax[3],
                                    float velRange, unsigned long long seed,
                                    uint maxAttempts) {
  u64 s = seed;
  std::vector<float> radii(radiiIn, radiiIn + n);
  float rMax = 0.0f, rMedian = 0.0f;
  for (uint i = 0; i < n; ++i) rMax = std::max(rMax, radii[i]);
  if (n) {
    std::vector<float> tmp(radii);
    std::nth_element(tmp.begin(), tmp.begin() + n / 2, tmp.end());
    rMedian = tmp[n / 2];
  }
  // The box is filled slab by slab along z, each slab at least 8 rMax thick
  // and given a share of the spheres proportional to the height its centres
  // can use, largest first; a candidate is then tested only against spheres
  // that are still in cache.  Centres of a slab lie inside it; its spheres
  // may reach into the previous slab and are tested against it.
  const float height = boxMax[2] - boxMin[2];
  uint slabs = (uint)std::max(1.0f, std::floor(height / (8.0f * rMax)));
  slabs = std::max(1u, std::min(slabs, n / 4096u + 1u));
  const float zs = height / (float)slabs;
  std::vector<double> weight(slabs);
  double wsum = 0.0;
  for (uint k = 0; k < slabs; ++k) {
    double lo = std::max((double)boxMin[2] + zs * k, (double)boxMin[2] + rMedian);
    double hi = std::min((double)boxMin[2] + zs * (k + 1), (double)boxMax[2] - rMedian);
    weight[k] = std::max(0.0, hi - lo);
    wsum += weight[k];
  }
  std::vector<size_t> first(slabs + 1, 0);
  double acc = 0.0;
  for (uint k = 0; k < slabs; ++k) {
    acc += weight[k];
    first[k + 1] = (k + 1 == slabs) ? n : (size_t)std::llround(acc / wsum * n);
  }
  for (uint k = 0; k < slabs; ++k)
    std::sort(radii.begin() + first[k], radii.begin() + first[k + 1],
              [](float a, float c) { return a > c; });

  // Occupancy grid with cell = 2 rMax: overlaps of a candidate are among the
  // 27 cells around it.
  const float cell = 2.0f * rMax;
  int dims[3];
  for (int k = 0; k < 3; ++k)
    dims[k] = std::max(1, (int)std::ceil((boxMax[k] - boxMin[k]) / cell));
  const size_t ncell = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<int> head(ncell, -1), next(n, -1);
  auto cellOf = [&](const float p[3], int c[3]) {
    for (int k = 0; k < 3; ++k) {
      int v = (int)std::floor((p[k] - boxMin[k]) / cell);
      c[k] = std::min(std::max(v, 0), dims[k] - 1);
    }
  };
  uint placed = 0;
  for (uint i = 0; i < n; ++i) {
    const float r = radii[i];
    uint slab = 0;
    while (slab + 1 < slabs && i >= first[slab + 1]) ++slab;
    float zlo = std::max(boxMin[2] + r, boxMin[2] + zs * (float)slab);
    float zhi = std::min(boxMax[2] - r, boxMin[2] + zs * (float)(slab + 1));
    if (zhi < zlo) zhi = zlo;
    bool ok = false;
    float p[3];
    for (uint a = 0; a < maxAttempts && !ok; ++a) {
      for (int k = 0; k < 2; ++k) {
        float lo = boxMin[k] + r, hi = boxMax[k] - r;
        p[k] = lo + uniformF(s) * (hi - lo);
      }
      p[2] = zlo + uniformF(s) * (zhi - zlo);
      int c[3];
      cellOf(p, c);
      ok = true;
      for (int dz = -1; dz <= 1 && ok; ++dz)
        for (int dy = -1; dy <= 1 && ok; ++dy)
          for (int dx = -1; dx <= 1 && ok; ++dx) {
            int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
            if (x < 0 || y < 0 || z < 0 || x >= dims[0] || y >= dims[1] || z >= dims[2])
              continue;
            for (int j = head[((size_t)z * dims[1] + y) * dims[0] + x]; j >= 0; j = next[j]) {
              const float *q = pos4 + 4 * (size_t)j;
              float ex = q[0] - p[0], ey = q[1] - p[1], ez = q[2] - p[2];
              float rr = q[3] + r;
              if (ex * ex + ey * ey + ez * ez < rr * rr) { ok = false; break; }
            }
          }
    }
    if (!ok) break;
    float *o = pos4 + 4 * (size_t)i;
    o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = r;
    for (int k = 0; k < 3; ++k) vel4[4 * (size_t)i + k] = (uniformF(s) * 2.0f - 1.0f) * velRange;
    vel4[4 * (size_t)i + 3] = 0.0f;
    int c[3];
    cellOf(p, c);
    size_t ci = ((size_t)c[2] * dims[1] + c[1]) * dims[0] + c[0];
    next[i] = head[ci];
    head[ci] = (int)i;
    placed = i + 1;
  }
  return placed;
}

