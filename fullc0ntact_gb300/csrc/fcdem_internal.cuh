// fcdem_internal.cuh -- shared declarations of the libfcdem translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fcdem.h"

namespace fcdem {

static_assert(sizeof(SimParams) == 104, "SimParams must keep the reference layout");
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
  unsigned *dStatus = nullptr;  // one device word of kStatus* bits
  void *scratch = nullptr;      // grown on demand, never shrunk
  size_t scratchBytes = 0;
};

// The context of the calling thread's current device (created on first use).
Context &ctx();
// The context of the current device if one has been created, else nullptr;
// never creates one (creating one allocates its device status word).
const Context *ctxIfCreated();
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

// collide (particles_kernel.cu:185-293), defined in fcdem_collide.cu.
// mode 0: newVel[index[i]] = (v + F, 0).  mode 1: also the next update's
// integrate and calcHash (posOut, hashOut).  force != nullptr also stores F.
void launchCollide(int mode, bool collider, float4 *newVel, float3 *force,
                   const float4 *sp, const float4 *sv, const unsigned *index,
                   const unsigned *cs, const unsigned *ce, unsigned n,
                   const KParams &kp, float4 *posOut, unsigned *hashOut, float dt);

}  // namespace fcdem
