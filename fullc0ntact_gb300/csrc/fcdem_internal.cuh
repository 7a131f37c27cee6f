// fcdem_internal.cuh -- shared declarations of the libfcdem translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fcdem.h"

namespace fcdem {

static_assert(sizeof(SimParams) == 104, "SimParams must keep the reference layout");
static_assert(sizeof(fcdemRigidBody) == 40, "fcdemRigidBody keeps i3d::Rbody<float>'s fields");
static_assert(offsetof(SimParams, colliderRadius) == 12, "layout");
static_assert(offsetof(SimParams, gravity) == 16, "layout");
static_assert(offsetof(SimParams, globalDamping) == 28, "layout");
static_assert(offsetof(SimParams, particleRadius) == 32, "layout");
static_assert(offsetof(SimParams, gridSize) == 36, "layout");
static_assert(offsetof(SimParams, numCells) == 48, "layout");
static_assert(offsetof(SimParams, worldOrigin) == 52, "layout");
static_assert(offsetof(SimParams, cellSize) == 64, "layout");
static_assert(offsetof(SimParams, numBodies) == 76, "layout");
static_assert(offsetof(SimParams, maxParticlesPerCell) == 80, "layout");
static_assert(offsetof(SimParams, spring) == 84, "layout");
static_assert(offsetof(SimParams, damping) == 88, "layout");
static_assert(offsetof(SimParams, shear) == 92, "layout");
static_assert(offsetof(SimParams, attraction) == 96, "layout");
static_assert(offsetof(SimParams, boundaryDamping) == 100, "layout");

// Device status bits (written by kernels with atomicOr, read by
// fcdemGetLastError).
enum : unsigned {
  kStatusTimeout = 1u,   // a bounded spin-wait gave up
  kStatusKeyRange = 2u,  // a sort key had bits above the sorted width
  kStatusRadiusBound = 4u,  // radius-from-w mode: a radius above particleRadius
  kStatusCellOverflow = 8u,  // counting sort: the list of crowded cells overflowed
};

// Everything a kernel needs from the parameter block, passed by value so
// that every launch carries its own copy (no __constant__ upload, and graph
// capture records the values).
struct KParams {
  SimParams p;
  int radiusFromW;
};

// Per-device library state.
struct Context {
  int device = -1;
  bool haveParams = false;
  SimParams params{};
  int radiusFromW = 0;
  int morton = 0;               // fcdemSetCellOrder
  unsigned *dStatus = nullptr;  // one device word of kStatus* bits
  void *scratch = nullptr;      // grown on demand, never shrunk
  size_t scratchBytes = 0;
  void *countBuf = nullptr;     // counting-sort pipeline of fcdemUpdate
  size_t countBytes = 0;
  unsigned countCells = 0;
  void *crowdBuf = nullptr;     // collide: groups of crowded particles
  unsigned crowdCap = 0;        // particles the group list covers
};

// The context of the calling thread's current device (created on first use).
Context &ctx();
// Copies the parameter block last given to setParameters on the current
// device (read under the context lock) and returns true; false when there is
// none.  Never creates a context (creating one allocates its status word).
bool paramsIfSet(SimParams &out);
// Multiprocessor count of the current device (queried once per device).
unsigned numSms();
// Look-back rounds a sort tile may make before it gives up
// (fcdemSetSortWaitLimit; default kSortWaitRounds).
unsigned sortWaitLimit();
// The status word of the allocation-free sort on the current device, or
// nullptr when that sort has not been set up there (fcdem_sort.cu).
unsigned *noAllocStatusWord();
// The stream this host thread issues work on (fcdemSetStream; default: the
// legacy default stream, as the reference).
cudaStream_t curStream();

// Records `code` as the pending error if none is pending.
void setError(int code);
// Records FCDEM_ERR_CUDA (and clears the CUDA error) when e != cudaSuccess.
bool cudaOk(cudaError_t e);
// Checks (and counts) the launch that was just issued.
bool launchOk();

// Stage profiling of fcdemUpdate (fcdemSetProfiling): brackets a stage with a
// CUDA event pair when profiling is on.
void stageBegin(int stage);
void stageEnd(int stage);
// Returns scratch of at least `bytes` bytes (256-byte aligned) or nullptr.
void *scratch(Context &c, size_t bytes);

KParams kparams(const Context &c);
// Morton cell keys need a cubic power-of-two grid of at most 1024 cells a side.
// The library's parameter copy marks Morton order with this value in
// maxParticlesPerCell (unused by the reference); see gridHash.
constexpr unsigned kMortonTag = 0x4d4f5254u;
bool mortonUsable(const SimParams &p);

// Number of key bits a sort must cover for keys below numCells.
inline int keyBits(unsigned numCells) {
  if (numCells <= 1u) return 1;
  unsigned m = numCells - 1u;
  int b = 0;
  while (m) { ++b; m >>= 1; }
  return b;
}

// Radix sort of (key, value) pairs, stable, ascending, in place, on the
// calling thread's stream.  Only the low `bits` key bits are sorted; keys
// with higher bits set raise kStatusKeyRange.  identityVals: the input values
// are 0..n-1 and are not read.  Defined in fcdem_sort.cu.
void radixSortPairs(Context &c, unsigned *keys, unsigned *vals, unsigned n,
                    int bits, bool identityVals = false);

// Cell-table fill (cellStart = 0xffffffff).  Defined in fcdem_stages.cu.
void fillU32(Context &c, unsigned *p, size_t count, unsigned value);
// The stage kernels with an explicit parameter block, on the current stream
// (fcdem_stages.cu): integrate (particles_kernel.cu:39-75), calcHash
// (:97-115), and the reorder with cell-range detection (:119-182; the cell
// tables must have been filled with 0xffffffff first).
void launchIntegrate(float4 *pos, float4 *vel, float dt, unsigned n, const KParams &kp);
void launchCalcHash(unsigned *hash, unsigned *index, const float4 *pos, unsigned n,
                    const KParams &kp);
void launchReorder(unsigned *cellStart, unsigned *cellEnd, float4 *sortedPos,
                   float4 *sortedVel, const unsigned *hash, const unsigned *index,
                   const float4 *oldPos, const float4 *oldVel, unsigned n, unsigned numCells);

// The cell ranges collide reads: either the reference's cellStart/cellEnd
// pair (empty = 0xffffffff start), or a prefix table off[] over numCells + 1
// cells (cell c = off[c] .. off[c+1]).
struct CellRanges {
  const unsigned *start = nullptr;
  const unsigned *end = nullptr;
  const unsigned *off = nullptr;
};

// What collide writes besides newVel (particles_kernel.cu:185-293 writes
// only newVel[index[i]] = (v + F, 0)).
struct CollideOut {
  float3 *force = nullptr;     // F per particle (original order), optional
  float4 *posOut = nullptr;    // mode 1/2: next-step integrated positions
  unsigned *hashOut = nullptr; // mode 1/2: next-step cell hashes
  unsigned *rankOut = nullptr; // mode 2: rank of the particle in its cell count
  unsigned *cnt = nullptr;     // mode 2: per-cell counters (atomic)
  unsigned *tileCnt = nullptr; // mode 2: per-4096-cell-tile counters (atomic)
  float dt = 0.0f;
};

// collide, defined in fcdem_collide.cu.  mode 0: the reference's output.
// mode 1: also the next update's integrate and calcHash.  mode 2 (counting
// pipeline): the next update's integrate and calcHash, written at the
// particle's sorted slot i (posOut[i], newVel[i], hashOut[i]) with its count
// rank (rankOut[i]) -- the state stays in sorted order between fused steps.
// mode 3 (last fused step): as 0, plus posOut[index[i]] = the position.
void launchCollide(int mode, bool collider, float4 *newVel, const float4 *sp,
                   const float4 *sv, const unsigned *index, const CellRanges &cells,
                   unsigned n, const KParams &kp, const CollideOut &out);

// One scene of a batch (fcdem_batch.cu), on the device.
struct BatchScene {
  SimParams p;
  float lo[3], hi[3];     // the scene's box (integrate clamps to it)
  unsigned cellBase;      // global id of the scene's cell 0
  unsigned particleBase;  // first particle of the scene
  int cull;               // collide may cull cells (see launchCollide)
  int shape;              // the scene's obstacle (index into the batch's maps), -1: none
};

// Batched collide: particles of many scenes in one launch; sceneOf[i] is
// the scene of particle/slot i, cell ids are cellBase + local hash.  mode 2
// (next integrate in the scene's box + hash + count at slot i) or 3 (last).
void launchCollideBatch(int mode, bool radiusFromW, const BatchScene *scenes,
                        const unsigned *sceneOf, float4 *newVel, const float4 *sp,
                        const float4 *sv, const unsigned *index, const unsigned *off,
                        unsigned n, const CollideOut &out);

// The counting-sort pipeline of fcdemUpdate (fcdem_count.cu).
struct CountBuffers {
  unsigned *cnt, *off, *rank, *slotKey, *slotIdx, *slotPrev;
  unsigned *tileCnt, *tileOff;  // per 4096-cell tile: counts and their prefix
  unsigned *tileOffPrev;        // per tile: the constant its offsets hold, or 0xffffffff
  unsigned *large;              // [0] = count, [1..largeCap] = cells too full for the re-rank
  unsigned *tileBlockSum;       // per 1024 tiles: their total (many-tile scans)
  unsigned *bitmaps;            // kFixupLarge: per-CTA bitmap + word prefix of particle indices
  unsigned scanTiles, largeCap;
};
bool countPipelineBegin(Context &c, float4 *pos, float4 *vel, float dt, unsigned *hash,
                        unsigned n, unsigned numCells, const KParams &kp, CountBuffers &b);
// Buffers over explicit storage (a batch owns its own); cnt/tileCnt must be
// zero on first use.
bool countBuffersIn(void *&buf, size_t &bytes, unsigned &cells, unsigned n, unsigned numCells,
                    CountBuffers &b);
// First step of a batch: integrate in each scene's box + hash + count.
bool countPipelineBeginBatch(const BatchScene *scenes, const unsigned *sceneOf, bool radiusFromW,
                             float4 *pos, float4 *vel, float dt, unsigned *hash, unsigned n,
                             unsigned numCells, const CountBuffers &b);
bool countPipelineSort(Context &c, const CountBuffers &b, const unsigned *origOf,
                       const float4 *prevPos, const float4 *prevVel, unsigned *hash,
                       unsigned *index, float4 *sortedPos, float4 *sortedVel, unsigned n,
                       unsigned numCells);
bool countPipelineTables(const CountBuffers &b, unsigned *cellStart, unsigned *cellEnd,
                         unsigned numCells);


// Unified-memory (particledem_um) step on the counting pipeline: the
// integrate with the distance-map boundary also writes the next step's
// calcHash and cell count (UmCount; nullptr on the last step).
struct UmCount {
  unsigned *hash, *rank, *cnt, *tileCnt;
};
// calcHash + count of the current positions (the first step).
bool umHashCount(const float4 *pos, unsigned n, const KParams &kp, const UmCount &count);
// d_integrateSystem + d_checkBoundaryDistMap, exact map query (map may be
// nullptr: no obstacle).
bool mapIntegrate(float4 *pos, float4 *vel, float dt, unsigned n, const KParams &kp,
                  const fcdemDistanceMap *map, const UmCount *count);
// Batch step with obstacles (fcdem_sdf.cu): for particle / slot i of scene
// sceneOf[i], the integrate in the scene's box with the contact of its
// obstacle maps[scenes[.].shape] between the velocity/position update and the
// box clamp; the map query culled by `net` where it predicts more than
// `skin` (net == nullptr: every in-box particle queries the map).  Reads
// inPos[i], vel[i]; writes pos[i], vel[i] and, with count, the next hash and
// count.  exact (optional) counts the exact queries.
struct MapView;
bool batchObstacleIntegrate(const BatchScene *scenes, const unsigned *sceneOf, bool radiusFromW,
                            const MapView *maps, fcdemSdfNet *net, float skin,
                            const float4 *inPos, float4 *pos, float4 *vel, float dt,
                            unsigned n, const UmCount *count, unsigned *exact, unsigned step);
// The same with the neural-SDF culling of the map query (fcdem_sdf.cu).
// The network's per-tile culling hints for `tiles` tiles, allocated (and
// cleared) when they grow; nullptr when they cannot be had.
unsigned char *sdfHints(fcdemSdfNet *net, unsigned tiles);
// The per-tile arrays of the network's culling per tile (when that is on)
// for n slots, grown now; false when they cannot be had.
bool sdfPrepareTiles(fcdemSdfNet *net, unsigned n);
// Changes with every change of the network's weights or normalisation (a
// recorded graph holds the values of its recording).
unsigned sdfVersion(const fcdemSdfNet *net);
// `step` (the step's number within a call) chooses the refresh steps of the
// per-tile culling hints; -1: a lone call, no hints.
bool sdfIntegrate(fcdemSdfNet *net, float4 *pos, float4 *vel, float dt, unsigned n,
                  const KParams &kp, const fcdemDistanceMap *map, float skin, unsigned *exact,
                  const UmCount *count, int step);

}  // namespace fcdem
