/*
 * refhost.cpp -- TEST INFRASTRUCTURE.  Builds the reference's own kernel
 * file (cuda_addon/particles_kernel.cu, included from the reference tree at
 * build time, never copied) as host code, and drives it with the launch glue
 * of cuda_addon/particleSystem.cu:135-270 restated: 256 threads per block for
 * calcHash and reorder, 64 for collide, cellStart memset to 0xff before the
 * reorder, a stable sort of (hash, index) for sortParticles.
 *
 * Threads of a block run one after another in ascending threadIdx order.  The
 * only kernel with a barrier (reorderDataAndFindCellStartD) reads
 * sharedHash[threadIdx] after the barrier, which thread threadIdx-1 (or thread
 * 0 itself) wrote before it, so ascending sequential order gives the same
 * values as a real launch.
 */
#include "host_prelude.h"
#include "particles_kernel.cu"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

static void grid_size(uint n, uint block, uint &nb, uint &nt) {
  nt = std::min(block, n);
  nb = nt ? (n + nt - 1) / nt : 0;
}

extern "C" {

unsigned fcref_sizeof_simparams(void) { return (unsigned)sizeof(SimParams); }

void fcref_setParameters(const void *hostParams) {
  std::memcpy(&params, hostParams, sizeof(SimParams));
}

/* particleSystem.cu:141-153: thrust::for_each over zip(pos4, vel4). */
void fcref_integrateSystem(float *pos, float *vel, float deltaTime,
                           uint numParticles) {
  float4 *p = (float4 *)pos, *v = (float4 *)vel;
  integrate_functor f(deltaTime);
  for (uint i = 0; i < numParticles; ++i) {
    std::tuple<float4 &, float4 &> t(p[i], v[i]);
    f(t);
  }
}

void fcref_calcHash(uint *hash, uint *index, float *pos, int numParticles) {
  uint nb, nt;
  grid_size((uint)numParticles, 256, nb, nt);
  blockDim = dim3(nt, 1, 1);
  for (uint b = 0; b < nb; ++b)
    for (uint t = 0; t < nt; ++t) {
      blockIdx.x = b;
      threadIdx.x = t;
      calcHashD(hash, index, (float4 *)pos, (uint)numParticles);
    }
}

/* thrust::sort_by_key on uint keys dispatches to a stable radix sort; the
 * ordering it defines (ascending key, ties in input order) is restated with
 * std::stable_sort. */
void fcref_sortParticles(uint *hash, uint *index, uint numParticles) {
  std::vector<uint> order(numParticles);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint a, uint b) { return hash[a] < hash[b]; });
  std::vector<uint> h(numParticles), x(numParticles);
  for (uint i = 0; i < numParticles; ++i) {
    h[i] = hash[order[i]];
    x[i] = index[order[i]];
  }
  std::copy(h.begin(), h.end(), hash);
  std::copy(x.begin(), x.end(), index);
}

void fcref_reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd,
                                       float *sortedPos, float *sortedVel,
                                       uint *hash, uint *index, float *oldPos,
                                       float *oldVel, uint numParticles,
                                       uint numCells) {
  uint nb, nt;
  grid_size(numParticles, 256, nb, nt);
  std::memset(cellStart, 0xff, numCells * sizeof(uint));
  blockDim = dim3(nt, 1, 1);
  for (uint b = 0; b < nb; ++b)
    for (uint t = 0; t < nt; ++t) {
      blockIdx.x = b;
      threadIdx.x = t;
      reorderDataAndFindCellStartD(cellStart, cellEnd, (float4 *)sortedPos,
                                   (float4 *)sortedVel, hash, index,
                                   (float4 *)oldPos, (float4 *)oldVel,
                                   numParticles);
    }
}

void fcref_collide(float *newVel, float *sortedPos, float *sortedVel,
                   uint *index, uint *cellStart, uint *cellEnd,
                   uint numParticles, uint numCells) {
  (void)numCells;
  uint nb, nt;
  grid_size(numParticles, 64, nb, nt);
  blockDim = dim3(nt, 1, 1);
  for (uint b = 0; b < nb; ++b)
    for (uint t = 0; t < nt; ++t) {
      blockIdx.x = b;
      threadIdx.x = t;
      collideD((float4 *)newVel, (float4 *)sortedPos, (float4 *)sortedVel,
               index, cellStart, cellEnd, numParticles);
    }
}

}  // extern "C"
