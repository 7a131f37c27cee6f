// fcdem_batch.cu -- many independent scenes stepped together.
//
// The reference steps one particle system at a time (ParticleSystem::update).
// A batch concatenates the particles of many scenes of uneven size and gives
// every scene its own parameter block, box and grid; the cells of all scenes
// share one id space (scene s owns ids cellBase[s] .. cellBase[s+1]).  One
// counting sort then orders all particles at once -- each scene's particles
// stay inside the scene's own slot range -- and each stage is one launch over
// every particle of every scene, whatever their sizes.  The whole multi-step
// sequence can be recorded once as a CUDA graph and replayed.
#include <cstring>
#include <vector>

#include "fcdem_map.cuh"

struct fcdemBatch {
  int device = -1;
  unsigned numScenes = 0, n = 0, numCells = 0;
  bool radiusFromW = false;
  fcdem::BatchScene *scenes = nullptr;  // device
  unsigned *sceneOf = nullptr;          // device, one per particle
  float4 *sortedPos = nullptr, *sortedVel = nullptr;
  unsigned *hash = nullptr, *index = nullptr;
  void *countBuf = nullptr;
  size_t countBytes = 0;
  unsigned countCells = 0;
  std::vector<unsigned> particleBase;  // host copy, numScenes + 1
  // recorded graph and what it was recorded for
  cudaGraphExec_t exec = nullptr;
  cudaStream_t captureStream = nullptr;
  const void *gPos = nullptr, *gVel = nullptr;
  float gDt = 0.0f;
  unsigned gSteps = 0;
  unsigned gNetVersion = 0;  // the network's version when the graph was recorded
  // obstacles (fcdemBatchSetObstacles)
  std::vector<fcdem::BatchScene> hostScenes;
  fcdem::MapView *maps = nullptr;  // device, one per shape
  fcdemSdfNet *net = nullptr;
  float skin = 0.0f;
  unsigned *exact = nullptr;  // device counter of exact map queries
};

namespace fcdem {
namespace {

bool pow2(unsigned g) { return g && !(g & (g - 1)); }

void freeBatch(fcdemBatch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->captureStream) cudaStreamDestroy(b->captureStream);
  cudaFree(b->scenes);
  cudaFree(b->sceneOf);
  cudaFree(b->sortedPos);
  cudaFree(b->sortedVel);
  cudaFree(b->hash);
  cudaFree(b->index);
  cudaFree(b->countBuf);
  cudaFree(b->maps);
  cudaFree(b->exact);
  delete b;
}

// The multi-step sequence on the current stream.
// With obstacles: the first integrate (particle order) with the obstacle
// contact, then per step the counting sort and a collide that leaves the new
// velocity at slot i, followed by the obstacle integrate in slot order with
// the next hash and count; the last collide writes the state back in
// particle order.
bool runBatchObstacles(fcdemBatch *b, const CountBuffers &cb, float4 *pos, float4 *vel,
                       float dt, unsigned steps) {
  Context &c = ctx();
  const UmCount count{b->hash, cb.rank, cb.cnt, cb.tileCnt};
  if (!batchObstacleIntegrate(b->scenes, b->sceneOf, b->radiusFromW, b->maps, b->net, b->skin,
                              pos, pos, vel, dt, b->n, &count, b->exact, 0))
    return false;
  for (unsigned s = 0; s < steps; ++s) {
    if (!countPipelineSort(c, cb, s == 0 ? nullptr : b->index, pos, vel, b->hash, b->index,
                           b->sortedPos, b->sortedVel, b->n, b->numCells))
      return false;
    const bool last = (s + 1 == steps);
    CollideOut out;
    out.posOut = pos;
    launchCollideBatch(last ? 3 : 4, b->radiusFromW, b->scenes, b->sceneOf, vel, b->sortedPos,
                       b->sortedVel, b->index, cb.off, b->n, out);
    if (!last &&
        !batchObstacleIntegrate(b->scenes, b->sceneOf, b->radiusFromW, b->maps, b->net, b->skin,
                                b->sortedPos, pos, vel, dt, b->n, &count, b->exact, s + 1))
      return false;
  }
  return true;
}

bool runBatch(fcdemBatch *b, float4 *pos, float4 *vel, float dt, unsigned steps) {
  Context &c = ctx();
  CountBuffers cb;
  if (!countBuffersIn(b->countBuf, b->countBytes, b->countCells, b->n, b->numCells, cb))
    return false;
  if (b->maps) return runBatchObstacles(b, cb, pos, vel, dt, steps);
  if (!countPipelineBeginBatch(b->scenes, b->sceneOf, b->radiusFromW, pos, vel, dt, b->hash,
                               b->n, b->numCells, cb))
    return false;
  for (unsigned s = 0; s < steps; ++s) {
    if (!countPipelineSort(c, cb, s == 0 ? nullptr : b->index, pos, vel, b->hash, b->index,
                           b->sortedPos, b->sortedVel, b->n, b->numCells))
      return false;
    const bool last = (s + 1 == steps);
    CollideOut out;
    out.posOut = pos;
    if (!last) {
      out.hashOut = b->hash;
      out.rankOut = cb.rank;
      out.cnt = cb.cnt;
      out.tileCnt = cb.tileCnt;
      out.dt = dt;
    }
    launchCollideBatch(last ? 3 : 2, b->radiusFromW, b->scenes, b->sceneOf, vel, b->sortedPos,
                       b->sortedVel, b->index, cb.off, b->n, out);
  }
  return true;
}

}  // namespace
}  // namespace fcdem

using namespace fcdem;

extern "C" {

fcdemBatch *fcdemBatchCreate(const fcdemBatchScene *scenes, uint numScenes, int radiusFromW) {
  if (!scenes || numScenes == 0) { setError(FCDEM_ERR_INVALID_VALUE); return nullptr; }
  fcdemBatch *b = new fcdemBatch();
  cudaGetDevice(&b->device);
  b->numScenes = numScenes;
  b->radiusFromW = radiusFromW != 0;
  std::vector<BatchScene> hs(numScenes);
  unsigned long long cellBase = 0, particleBase = 0;
  b->particleBase.resize(numScenes + 1);
  for (uint s = 0; s < numScenes; ++s) {
    const fcdemBatchScene &in = scenes[s];
    const SimParams &p = in.params;
    unsigned long long cells = 1;
    for (int k = 0; k < 3; ++k) {
      if (!pow2(p.gridSize[k])) { setError(FCDEM_ERR_INVALID_VALUE); freeBatch(b); return nullptr; }
      cells *= p.gridSize[k];
    }
    BatchScene &d = hs[s];
    std::memset(&d, 0, sizeof(d));
    d.p = p;
    d.p.numCells = (unsigned)cells;
    d.p.maxParticlesPerCell = 0u;  // linear cell keys in a batch
    for (int k = 0; k < 3; ++k) {
      d.lo[k] = in.boxLo[k];
      d.hi[k] = in.boxHi[k];
    }
    d.shape = -1;
    d.cellBase = (unsigned)cellBase;
    d.particleBase = (unsigned)particleBase;
    const float minCell = fminf(p.cellSize[0], fminf(p.cellSize[1], p.cellSize[2]));
    d.cull = p.gridSize[0] >= 3 && p.gridSize[1] >= 3 && p.gridSize[2] >= 3 &&
             p.particleRadius > 0.0f && 2.0f * p.particleRadius <= minCell;
    b->particleBase[s] = (unsigned)particleBase;
    cellBase += cells;
    particleBase += in.numParticles;
  }
  b->particleBase[numScenes] = (unsigned)particleBase;
  if (cellBase >= (1ull << 32) - 1 || particleBase >= (1ull << 30)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    freeBatch(b);
    return nullptr;
  }
  b->n = (unsigned)particleBase;
  b->numCells = (unsigned)cellBase;
  std::vector<unsigned> sceneOf(b->n);
  for (uint s = 0; s < numScenes; ++s)
    for (unsigned i = b->particleBase[s]; i < b->particleBase[s + 1]; ++i) sceneOf[i] = s;
  const size_t n = b->n ? b->n : 1;
  bool ok = cudaMalloc(&b->scenes, sizeof(BatchScene) * numScenes) == cudaSuccess &&
            cudaMalloc(&b->sceneOf, 4 * n) == cudaSuccess &&
            cudaMalloc(&b->sortedPos, 16 * n) == cudaSuccess &&
            cudaMalloc(&b->sortedVel, 16 * n) == cudaSuccess &&
            cudaMalloc(&b->hash, 4 * n) == cudaSuccess &&
            cudaMalloc(&b->index, 4 * n) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    setError(FCDEM_ERR_ALLOC);
    freeBatch(b);
    return nullptr;
  }
  cudaOk(cudaMemcpy(b->scenes, hs.data(), sizeof(BatchScene) * numScenes,
                    cudaMemcpyHostToDevice));
  b->hostScenes = hs;
  if (b->n)
    cudaOk(cudaMemcpy(b->sceneOf, sceneOf.data(), 4 * (size_t)b->n, cudaMemcpyHostToDevice));
  CountBuffers cb;  // allocate now: recording a graph must not allocate
  if (!countBuffersIn(b->countBuf, b->countBytes, b->countCells, b->n, b->numCells, cb)) {
    freeBatch(b);
    return nullptr;
  }
  ctx();  // the library context (status word) too
  return b;
}

void fcdemBatchDestroy(fcdemBatch *b) { freeBatch(b); }

void fcdemBatchSetObstacles(fcdemBatch *b, const fcdemDistanceMap *const *maps, uint numMaps,
                            const int *sceneShape, fcdemSdfNet *net, float skin) {
  if (!b || (numMaps && (!maps || !sceneShape)) || (net && !(skin >= 0.0f))) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  for (uint k = 0; k < numMaps; ++k)
    if (!maps[k]) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (numMaps)
    for (uint s = 0; s < b->numScenes; ++s)
      if (sceneShape[s] < -1 || sceneShape[s] >= (int)numMaps) {
        setError(FCDEM_ERR_INVALID_VALUE);
        return;
      }
  if (!cudaOk(cudaDeviceSynchronize())) return;  // work in flight may read the old ones
  cudaFree(b->maps);
  b->maps = nullptr;
  if (b->exec) {  // a recorded graph holds the old pipeline
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  for (uint s = 0; s < b->numScenes; ++s)
    b->hostScenes[s].shape = numMaps ? sceneShape[s] : -1;
  if (!cudaOk(cudaMemcpy(b->scenes, b->hostScenes.data(), sizeof(BatchScene) * b->numScenes,
                         cudaMemcpyHostToDevice)))
    return;
  b->net = numMaps ? net : nullptr;
  b->skin = skin;
  if (numMaps == 0) return;
  if (net) {  // now, not while a graph is recorded
    sdfHints(net, (b->n + 127) / 128);
    sdfPrepareTiles(net, b->n);
  }
  std::vector<MapView> hv(numMaps);
  for (uint k = 0; k < numMaps; ++k) hv[k] = view(maps[k]);
  if (cudaMalloc(&b->maps, sizeof(MapView) * numMaps) != cudaSuccess ||
      (!b->exact && cudaMalloc(&b->exact, sizeof(unsigned)) != cudaSuccess)) {
    cudaGetLastError();
    cudaFree(b->maps);
    b->maps = nullptr;
    setError(FCDEM_ERR_ALLOC);
    return;
  }
  cudaOk(cudaMemcpy(b->maps, hv.data(), sizeof(MapView) * numMaps, cudaMemcpyHostToDevice));
  cudaOk(cudaMemset(b->exact, 0, sizeof(unsigned)));
}

unsigned long long fcdemBatchExactQueries(fcdemBatch *b, int reset) {
  if (!b) { setError(FCDEM_ERR_INVALID_VALUE); return 0; }
  if (!b->exact) return 0;
  unsigned v = 0;
  if (!cudaOk(cudaDeviceSynchronize()) ||
      !cudaOk(cudaMemcpy(&v, b->exact, sizeof(unsigned), cudaMemcpyDeviceToHost)))
    return 0;
  if (reset) cudaOk(cudaMemset(b->exact, 0, sizeof(unsigned)));
  return v;
}

uint fcdemBatchNumParticles(const fcdemBatch *b) { return b ? b->n : 0u; }
uint fcdemBatchNumCells(const fcdemBatch *b) { return b ? b->numCells : 0u; }

void fcdemBatchUpdate(fcdemBatch *b, float *pos, float *vel, float deltaTime, uint steps,
                      int useGraph) {
  if (!b || !pos || !vel) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (steps == 0 || b->n == 0) return;
  if (!useGraph) {
    runBatch(b, (float4 *)pos, (float4 *)vel, deltaTime, steps);
    return;
  }
  // the network's normalisation and BF16 weights are recorded by value: a
  // retrained network needs a new recording
  const bool same = b->exec && b->gPos == pos && b->gVel == vel && b->gDt == deltaTime &&
                    b->gSteps == steps && (!b->net || sdfVersion(b->net) == b->gNetVersion);
  if (!same) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    if (!b->captureStream &&
        !cudaOk(cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking)))
      return;
    // the network's per-tile arrays are grown now, not while the graph is
    // recorded (the culling mode may have changed since the obstacles were set)
    if (b->net && !sdfPrepareTiles(b->net, b->n)) return;
    const cudaStream_t prev = curStream();
    fcdemSetStream(b->captureStream);
    cudaGraph_t graph = nullptr;
    bool ok = cudaOk(cudaStreamBeginCapture(b->captureStream, cudaStreamCaptureModeThreadLocal));
    if (ok) {
      bool ran = runBatch(b, (float4 *)pos, (float4 *)vel, deltaTime, steps);
      ok = cudaOk(cudaStreamEndCapture(b->captureStream, &graph)) && ran;
    }
    fcdemSetStream(prev);
    if (!ok || !graph) {
      if (graph) cudaGraphDestroy(graph);
      setError(FCDEM_ERR_CUDA);
      return;
    }
    ok = cudaOk(cudaGraphInstantiate(&b->exec, graph, 0));
    cudaGraphDestroy(graph);
    if (!ok) return;
    b->gPos = pos;
    b->gVel = vel;
    b->gDt = deltaTime;
    b->gSteps = steps;
    b->gNetVersion = sdfVersion(b->net);
  }
  cudaOk(cudaGraphLaunch(b->exec, curStream()));
}

}  // extern "C"
