// fcdem_stages.cu -- integrate, hash, reorder and collide kernels and the
// reference-named entry points that launch them
// (particleSystem.cu:141-262, particles_kernel.cu:39-293).
#include "fcdem_dem.cuh"

namespace fcdem {

constexpr unsigned kEmpty = 0xffffffffu;

// ---------------------------------------------------------------------------
// integrate (particles_kernel.cu:39-75; launched by thrust::for_each in
// particleSystem.cu:141-153).  One thread per particle, 128-bit loads/stores.
__global__ void __launch_bounds__(256)
kIntegrate(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt,
           unsigned n, KParams kp) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  float r = kp.radiusFromW ? p4.w : kp.p.particleRadius;
  integrateOne(p, v, dt, r, kp.p);
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, v4.w);
}

// ---------------------------------------------------------------------------
// calcHash (particles_kernel.cu:97-115).
__global__ void __launch_bounds__(256)
kCalcHash(unsigned *__restrict__ hash, unsigned *__restrict__ index,
          const float4 *__restrict__ pos, unsigned n, KParams kp) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = ldg4(pos + i);
  int3 g = gridPos(p.x, p.y, p.z, kp.p);
  hash[i] = gridHash(g.x, g.y, g.z, kp.p);
  index[i] = i;
}

// integrate + calcHash in one pass (the first two stages of
// ParticleSystem::update, particleSystem.cpp:239-251).
__global__ void __launch_bounds__(256)
kIntegrateHash(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt,
               unsigned *__restrict__ hash, unsigned *__restrict__ index,
               unsigned n, KParams kp) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  float r = kp.radiusFromW ? p4.w : kp.p.particleRadius;
  integrateOne(p, v, dt, r, kp.p);
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, v4.w);
  int3 g = gridPos(p.x, p.y, p.z, kp.p);
  hash[i] = gridHash(g.x, g.y, g.z, kp.p);
  index[i] = i;
}

// ---------------------------------------------------------------------------
// Fill (the cudaMemset of particleSystem.cu:198).  16-byte stores where the
// pointer allows, grid-stride.
__global__ void __launch_bounds__(256)
kFill(unsigned *__restrict__ p, size_t count, unsigned value) {
  size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t head = (16u - ((uintptr_t)p & 15u)) / 4u & 3u;
  if (head > count) head = count;
  if (tid < head) p[tid] = value;
  size_t n4 = (count - head) / 4;
  uint4 *q = reinterpret_cast<uint4 *>(p + head);
  uint4 v = make_uint4(value, value, value, value);
  for (size_t k = tid; k < n4; k += stride) q[k] = v;
  size_t tail = head + n4 * 4;
  if (tid < count - tail) p[tail + tid] = value;
}

void fillU32(Context &, unsigned *p, size_t count, unsigned value) {
  if (count == 0) return;
  size_t work = (count + 3) / 4;
  unsigned blocks = (unsigned)((work + 255) / 256);
  if (blocks > numSms() * 16u) blocks = numSms() * 16u;
  if (blocks == 0) blocks = 1;
  kFill<<<blocks, 256, 0, curStream()>>>(p, count, value);
  launchOk();
}

// ---------------------------------------------------------------------------
// reorderDataAndFindCellStart (particles_kernel.cu:119-182).  The previous
// hash is read directly (adjacent threads share the cache line), the gathers
// are 128-bit.
__global__ void __launch_bounds__(256)
kReorder(unsigned *__restrict__ cellStart, unsigned *__restrict__ cellEnd,
         float4 *__restrict__ sortedPos, float4 *__restrict__ sortedVel,
         const unsigned *__restrict__ hash, const unsigned *__restrict__ index,
         const float4 *__restrict__ oldPos, const float4 *__restrict__ oldVel,
         unsigned n, unsigned numCells, unsigned *status) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned h = __ldg(hash + i);
  unsigned s = __ldg(index + i);
  // Hashes come from calcHash and are below numCells, indices below n; a
  // caller's array that breaks this is reported instead of written through.
  if (h >= numCells || s >= n) {
    atomicOr(status, (unsigned)kStatusKeyRange);
    return;
  }
  if (i == 0) {
    cellStart[h] = 0;
  } else {
    unsigned hp = __ldg(hash + i - 1);
    if (h != hp) {
      cellStart[h] = i;
      if (hp < numCells) cellEnd[hp] = i;
    }
  }
  if (i == n - 1) cellEnd[h] = n;
  sortedPos[i] = ldg4(oldPos + s);
  sortedVel[i] = ldg4(oldVel + s);
}

// collide lives in fcdem_collide.cu (launchCollide).

void launchIntegrateHash(float4 *pos, float4 *vel, float dt, unsigned *hash,
                         unsigned *index, unsigned n, const KParams &kp) {
  if (n == 0) return;
  kIntegrateHash<<<(n + 255) / 256, 256, 0, curStream()>>>(pos, vel, dt, hash,
                                                           index, n, kp);
  launchOk();
}

void launchIntegrate(float4 *pos, float4 *vel, float dt, unsigned n, const KParams &kp) {
  if (n == 0) return;
  kIntegrate<<<(n + 255) / 256, 256, 0, curStream()>>>(pos, vel, dt, n, kp);
  launchOk();
}

void launchCalcHash(unsigned *hash, unsigned *index, const float4 *pos, unsigned n,
                    const KParams &kp) {
  if (n == 0) return;
  kCalcHash<<<(n + 255) / 256, 256, 0, curStream()>>>(hash, index, pos, n, kp);
  launchOk();
}

void launchReorder(unsigned *cellStart, unsigned *cellEnd, float4 *sortedPos,
                   float4 *sortedVel, const unsigned *hash,
                   const unsigned *index, const float4 *oldPos,
                   const float4 *oldVel, unsigned n, unsigned numCells) {
  if (n == 0) return;
  kReorder<<<(n + 255) / 256, 256, 0, curStream()>>>(
      cellStart, cellEnd, sortedPos, sortedVel, hash, index, oldPos, oldVel, n,
      numCells, ctx().dStatus);
  launchOk();
}

static bool gridOk(const SimParams &p) {
  unsigned long long cells = 1;
  for (int k = 0; k < 3; ++k) {
    unsigned g = p.gridSize[k];
    if (g == 0 || (g & (g - 1)) != 0) return false;
    cells *= g;
  }
  return cells <= p.numCells;  // every hash indexes the cell tables
}

// The cell tables the caller passes must cover every hash of the grid.
static bool tablesOk(const SimParams &p, unsigned numCells) {
  unsigned long long cells =
      (unsigned long long)p.gridSize[0] * p.gridSize[1] * p.gridSize[2];
  if (cells > numCells) { setError(FCDEM_ERR_INVALID_VALUE); return false; }
  return true;
}

// fcdemUpdate pipeline: 0 radix sort + reorder, 1 counting sort (default).
int g_updatePipeline = 1;

bool readyFor(const Context &c) {
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return false; }
  if (!gridOk(c.params)) { setError(FCDEM_ERR_INVALID_VALUE); return false; }
  return true;
}

}  // namespace fcdem

using namespace fcdem;

extern "C" {

void integrateSystem(float *pos, float *vel, float deltaTime, uint numParticles) {
  Context &c = ctx();
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return; }
  if (numParticles == 0) return;
  if (!pos || !vel) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  kIntegrate<<<(numParticles + 255) / 256, 256, 0, curStream()>>>(
      (float4 *)pos, (float4 *)vel, deltaTime, numParticles, kparams(c));
  launchOk();
}

void calcHash(uint *gridParticleHash, uint *gridParticleIndex, float *pos,
              int numParticles) {
  Context &c = ctx();
  if (!readyFor(c)) return;
  if (numParticles <= 0) {
    if (numParticles < 0) setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  if (!gridParticleHash || !gridParticleIndex || !pos) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  unsigned n = (unsigned)numParticles;
  kCalcHash<<<(n + 255) / 256, 256, 0, curStream()>>>(
      gridParticleHash, gridParticleIndex, (const float4 *)pos, n, kparams(c));
  launchOk();
}

void reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd,
                                 float *sortedPos, float *sortedVel,
                                 uint *gridParticleHash, uint *gridParticleIndex,
                                 float *oldPos, float *oldVel,
                                 uint numParticles, uint numCells) {
  Context &c = ctx();
  if (!cellStart || (numParticles && (!cellEnd || !sortedPos || !sortedVel ||
                                      !gridParticleHash || !gridParticleIndex ||
                                      !oldPos || !oldVel))) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  fillU32(c, cellStart, numCells, kEmpty);
  launchReorder(cellStart, cellEnd, (float4 *)sortedPos, (float4 *)sortedVel,
                gridParticleHash, gridParticleIndex, (const float4 *)oldPos,
                (const float4 *)oldVel, numParticles, numCells);
}

void collide(float *newVel, float *sortedPos, float *sortedVel,
             uint *gridParticleIndex, uint *cellStart, uint *cellEnd,
             uint numParticles, uint numCells) {
  Context &c = ctx();
  if (!readyFor(c) || !tablesOk(c.params, numCells)) return;
  if (numParticles == 0) return;
  if (!newVel || !sortedPos || !sortedVel || !gridParticleIndex || !cellStart ||
      !cellEnd) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  CellRanges cells;
  cells.start = cellStart;
  cells.end = cellEnd;
  launchCollide(0, true, (float4 *)newVel, (const float4 *)sortedPos,
                (const float4 *)sortedVel, gridParticleIndex, cells, numParticles,
                kparams(c), CollideOut());
}

void sortParticles(uint *dGridParticleHash, uint *dGridParticleIndex,
                   uint numParticles) {
  Context &c = ctx();
  if (numParticles < 2) return;
  if (!dGridParticleHash || !dGridParticleIndex) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  int bits = c.haveParams ? keyBits(c.params.numCells) : 32;
  radixSortPairs(c, dGridParticleHash, dGridParticleIndex, numParticles, bits);
}

void fcdemUpdate(float *pos, float *vel, float *sortedPos, float *sortedVel,
                 uint *hash, uint *index, uint *cellStart, uint *cellEnd,
                 float deltaTime, uint numParticles, uint numCells, uint steps) {
  Context &c = ctx();
  if (!readyFor(c) || !tablesOk(c.params, numCells)) return;
  if (steps == 0 || numParticles == 0) return;
  if (!pos || !vel || !sortedPos || !sortedVel || !hash || !index ||
      !cellStart || !cellEnd || numCells == 0) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  const KParams kp = kparams(c);
  const int bits = keyBits(c.params.numCells);
  const unsigned n = numParticles;
  if (g_updatePipeline == 1) {
    // Counting-sort pipeline (fcdem_count.cu).  Between fused steps the state
    // stays in the previous step's sorted order: collide writes the
    // integrated position/velocity, next hash and count rank of slot i at
    // entry i of pos/vel/hash/rank, and the next scatter and fix-up read them
    // in that order (near-sequential instead of random).  The first step
    // starts from particle order; the last collide writes vel and pos back in
    // particle order, and the cell tables are written once at the end.
    CountBuffers b;
    stageBegin(0);
    bool ok = countPipelineBegin(c, (float4 *)pos, (float4 *)vel, deltaTime, hash, n,
                                 numCells, kp, b);
    stageEnd(0);
    for (uint s = 0; ok && s < steps; ++s) {
      stageBegin(1);
      ok = countPipelineSort(c, b, s == 0 ? nullptr : index, (const float4 *)pos,
                             (const float4 *)vel, hash, index, (float4 *)sortedPos,
                             (float4 *)sortedVel, n, numCells);
      stageEnd(1);
      if (!ok) break;
      const bool last = (s + 1 == steps);
      CellRanges cells;
      cells.off = b.off;
      CollideOut out;
      out.posOut = (float4 *)pos;
      if (!last) {
        out.hashOut = hash;
        out.rankOut = b.rank;
        out.cnt = b.cnt;
        out.tileCnt = b.tileCnt;
        out.dt = deltaTime;
      }
      stageBegin(4);
      launchCollide(last ? 3 : 2, true, (float4 *)vel, (const float4 *)sortedPos,
                    (const float4 *)sortedVel, index, cells, n, kp, out);
      stageEnd(4);
    }
    if (ok) {
      stageBegin(2);
      countPipelineTables(b, cellStart, cellEnd, numCells);
      stageEnd(2);
    }
    return;
  }
  stageBegin(0);
  launchIntegrateHash((float4 *)pos, (float4 *)vel, deltaTime, hash, index, n, kp);
  stageEnd(0);
  for (uint s = 0; s < steps; ++s) {
    // After the first step the fused collide has written the keys but not
    // the identity index (see kCollide); the sort generates it.
    stageBegin(1);
    radixSortPairs(c, hash, index, n, bits, /*identityVals=*/s > 0);
    stageEnd(1);
    stageBegin(2);
    fillU32(c, cellStart, numCells, kEmpty);
    stageEnd(2);
    stageBegin(3);
    launchReorder(cellStart, cellEnd, (float4 *)sortedPos, (float4 *)sortedVel,
                  hash, index, (const float4 *)pos, (const float4 *)vel, n, numCells);
    stageEnd(3);
    const bool last = (s + 1 == steps);
    CellRanges cells;
    cells.start = cellStart;
    cells.end = cellEnd;
    CollideOut out;
    if (!last) {
      out.posOut = (float4 *)pos;
      out.hashOut = hash;
      out.dt = deltaTime;
    }
    stageBegin(4);
    launchCollide(last ? 0 : 1, true, (float4 *)vel, (const float4 *)sortedPos,
                  (const float4 *)sortedVel, index, cells, n, kp, out);
    stageEnd(4);
  }
}

void fcdemSetUpdatePipeline(int pipeline) { g_updatePipeline = pipeline == 0 ? 0 : 1; }

void fcdemUM_update(float *pos, float *vel, float *force, float *sortedPos, float *sortedVel,
                    uint *hash, uint *index, uint *cellStart, uint *cellEnd, float deltaTime,
                    uint numParticles, uint numCells, uint steps, const fcdemDistanceMap *map,
                    fcdemSdfNet *net, float skin, uint *exactQueries) {
  Context &c = ctx();
  if (!readyFor(c) || !tablesOk(c.params, numCells)) return;
  if (steps == 0 || numParticles == 0) return;
  if (!pos || !vel || !sortedPos || !sortedVel || !hash || !index || !cellStart || !cellEnd ||
      numCells == 0 || (net && (!map || !(skin >= 0.0f)))) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  const KParams kp = kparams(c);
  const unsigned n = numParticles;
  // Per step, as CollisionPipeline<dem_gpu_unified>::startPipeline
  // (dempipeline.hpp:113-120): calcHash, sortParticles, reorder, evalForces,
  // integrateSystem.  The sort is the counting pipeline from particle order
  // each step; evalForces writes vel (and force) in particle order; the
  // integrate also writes the next step's hash and count.
  CountBuffers b;
  if (!countBuffersIn(c.countBuf, c.countBytes, c.countCells, n, numCells, b)) return;
  const UmCount count{hash, b.rank, b.cnt, b.tileCnt};
  stageBegin(0);
  bool ok = umHashCount((const float4 *)pos, n, kp, count);
  stageEnd(0);
  for (uint s = 0; ok && s < steps; ++s) {
    stageBegin(1);
    ok = countPipelineSort(c, b, nullptr, (const float4 *)pos, (const float4 *)vel, hash, index,
                           (float4 *)sortedPos, (float4 *)sortedVel, n, numCells);
    stageEnd(1);
    if (!ok) break;
    CellRanges cells;
    cells.off = b.off;
    CollideOut out;
    out.force = (float3 *)force;
    stageBegin(4);
    launchCollide(0, false, (float4 *)vel, (const float4 *)sortedPos, (const float4 *)sortedVel,
                  index, cells, n, kp, out);
    stageEnd(4);
    const bool last = (s + 1 == steps);
    stageBegin(0);
    if (net)
      ok = sdfIntegrate(net, (float4 *)pos, (float4 *)vel, deltaTime, n, kp, map, skin,
                        exactQueries, last ? nullptr : &count, (int)s);
    else
      ok = mapIntegrate((float4 *)pos, (float4 *)vel, deltaTime, n, kp, map,
                        last ? nullptr : &count);
    stageEnd(0);
  }
  if (ok) {
    stageBegin(2);
    countPipelineTables(b, cellStart, cellEnd, numCells);
    stageEnd(2);
  }
}

}  // extern "C"
