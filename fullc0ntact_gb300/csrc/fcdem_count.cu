// fcdem_count.cu -- the cell counting-sort pipeline of fcdemUpdate.
//
// The reference re-sorts all particles by cell hash every step
// (thrust::sort_by_key, particleSystem.cu:328-333) and then scatters the
// cell ranges (reorderDataAndFindCellStartD).  Inside fcdemUpdate the same
// result comes from a counting sort over the cells:
//
//   count   the kernel that computes a particle's cell hash h (the fused
//           collide+integrate of the previous step, or kIntegrateHashCount)
//           also takes r = atomicAdd(&cnt[h], 1);
//   scan    kScanCells: off = exclusive prefix sum of cnt over C + 1 cells
//           (single pass, decoupled look-back), and cnt is cleared for the
//           next step; off[c] .. off[c+1] is cell c's range, empty or not;
//   scatter kScatterCells: slot off[h] + r receives (h, particle);
//   fix-up  kFixupGather: the atomic ranks order a cell's members
//           arbitrarily, so each slot re-ranks its particle among the
//           members of its cell by particle index (the order of the
//           reference's stable sort), then writes hash/index in sorted order
//           and gathers pos/vel into sortedPos/sortedVel (the reorder).
//
// The collide kernel reads `off` instead of cellStart/cellEnd.  At the end of
// fcdemUpdate kCellTables writes cellStart/cellEnd from `off`, so every array
// holds what the reference's stages leave.  Cells with more than
// kFixupMaxCell members keep the atomic order and raise kStatusCellOverflow
// (such a cell makes the reference's collide quadratic in it as well).
#include "fcdem_dem.cuh"

namespace fcdem {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096 cells
constexpr unsigned kFlagAgg = 1u << 30;
constexpr unsigned kFlagPrefix = 2u << 30;
constexpr unsigned kValueMask = (1u << 30) - 1u;
constexpr unsigned kSpinLimit = 1u << 22;
constexpr unsigned kEmpty = 0xffffffffu;

__device__ __forceinline__ unsigned ldVolatile(const unsigned *p) {
  return *(const volatile unsigned *)p;
}
__device__ __forceinline__ void stVolatile(unsigned *p, unsigned v) {
  *(volatile unsigned *)p = v;
}

// Exclusive prefix sum of cnt[0..m) into off[0..m), clearing cnt.  lookback
// (one word per tile) and *tileCounter must be zero on entry.
__global__ void __launch_bounds__(kScanThreads)
kScanCells(unsigned *__restrict__ cnt, unsigned *__restrict__ off, unsigned m,
           unsigned *lookback, unsigned *tileCounter, unsigned *status) {
  __shared__ unsigned sTile, sExcl;
  __shared__ unsigned sWarp[kScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sTile = atomicAdd(tileCounter, 1u);
  __syncthreads();
  const unsigned tile = sTile;
  const size_t base = (size_t)tile * kScanTile + (size_t)tid * kScanItems;
  unsigned v[kScanItems];
  unsigned sum = 0;
  // a thread owns kScanItems consecutive cells (16-byte loads when whole)
  if (base + kScanItems <= m && ((base & 3u) == 0)) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      uint4 t = reinterpret_cast<const uint4 *>(cnt + base)[q];
      v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) v[q] = base + q < m ? cnt[base + q] : 0u;
  }
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) sum += v[q];
  // block exclusive scan of the per-thread sums
  unsigned x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sWarp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned s = lane < kScanThreads / 32 ? sWarp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kScanThreads / 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) sWarp[lane] = s;
  }
  __syncthreads();
  const unsigned threadExcl = (warp ? sWarp[warp - 1] : 0u) + x - sum;
  const unsigned tileSum = sWarp[kScanThreads / 32 - 1];
  // decoupled look-back for the tile's exclusive prefix, warp 0 reading 32
  // predecessor tiles per round
  if (warp == 0) {
    unsigned excl = 0;
    if (tile == 0) {
      if (lane == 0) stVolatile(lookback, kFlagPrefix | (tileSum & kValueMask));
    } else {
      if (lane == 0) stVolatile(lookback + tile, kFlagAgg | (tileSum & kValueMask));
      int t = (int)tile - 1;  // newest tile of this round (lane 0)
      unsigned spins = 0;
      while (t >= 0) {
        const int mine = t - lane;
        unsigned w = mine >= 0 ? ldVolatile(lookback + mine) : (kFlagPrefix | 0u);
        unsigned flag = w & ~kValueMask;
        // wait while a tile before the closest inclusive prefix has not
        // published anything yet
        const unsigned preMask = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
        const unsigned zeroMask = __ballot_sync(0xffffffffu, flag == 0u);
        const unsigned relevant = preMask ? ((preMask & (0u - preMask)) - 1u) : 0xffffffffu;
        if (zeroMask & relevant) {
          if (++spins > kSpinLimit) {
            if (lane == 0) atomicOr(status, (unsigned)kStatusTimeout);
            break;
          }
          if (spins > 64) __nanosleep(64);
          continue;
        }
        // the closest lane holding an inclusive prefix ends the walk
        unsigned pre = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
        int stop = pre ? __ffs(pre) - 1 : 31;
        unsigned v = lane <= stop ? (w & kValueMask) : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (pre) break;
        t -= 32;
      }
      if (lane == 0) stVolatile(lookback + tile, kFlagPrefix | ((excl + tileSum) & kValueMask));
    }
    if (lane == 0) sExcl = excl;
  }
  __syncthreads();
  unsigned run = sExcl + threadExcl;
  unsigned o[kScanItems];
#pragma unroll
  for (int q = 0; q < kScanItems; ++q) {
    o[q] = run;
    run += v[q];
  }
  if (base + kScanItems <= m && ((base & 3u) == 0)) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      reinterpret_cast<uint4 *>(off + base)[q] = make_uint4(o[4 * q], o[4 * q + 1],
                                                            o[4 * q + 2], o[4 * q + 3]);
      reinterpret_cast<uint4 *>(cnt + base)[q] = make_uint4(0u, 0u, 0u, 0u);
    }
  } else {
#pragma unroll
    for (int q = 0; q < kScanItems; ++q)
      if (base + q < m) {
        off[base + q] = o[q];
        cnt[base + q] = 0u;
      }
  }
}

// Entry i (a slot of the previous order, or the particle itself on the first
// step) holds the particle's new cell hash h and its count rank r; slot
// off[h] + r receives the hash, the particle's index and the entry i.
__global__ void __launch_bounds__(256)
kScatterCells(const unsigned *__restrict__ hashN, const unsigned *__restrict__ rankN,
              const unsigned *__restrict__ origOf, const unsigned *__restrict__ off,
              unsigned *__restrict__ slotKey, unsigned *__restrict__ slotOrig,
              unsigned *__restrict__ slotPrev, unsigned n, unsigned numCells,
              unsigned *status) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned h = __ldg(hashN + i);
  if (h >= numCells) {
    atomicOr(status, (unsigned)kStatusKeyRange);
    return;
  }
  unsigned s = __ldg(off + h) + __ldg(rankN + i);
  if (s >= n) {
    atomicOr(status, (unsigned)kStatusKeyRange);
    return;
  }
  slotKey[s] = h;
  slotOrig[s] = origOf ? __ldg(origOf + i) : i;
  slotPrev[s] = i;
}

constexpr unsigned kFixupMaxCell = 4096;

// Stable order inside each cell + the reorder gather.  The particle of slot
// s is re-ranked among its cell's members by particle index; its position and
// velocity are gathered from entry slotPrev[s] of the previous order.
__global__ void __launch_bounds__(256)
kFixupGather(const unsigned *__restrict__ slotKey, const unsigned *__restrict__ slotOrig,
             const unsigned *__restrict__ slotPrev, const unsigned *__restrict__ off,
             unsigned *__restrict__ hashOut, unsigned *__restrict__ indexOut,
             float4 *__restrict__ sortedPos, float4 *__restrict__ sortedVel,
             const float4 *__restrict__ prevPos, const float4 *__restrict__ prevVel,
             unsigned n, unsigned numCells, unsigned *status) {
  unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const unsigned h = __ldg(slotKey + s);
  const unsigned me = __ldg(slotOrig + s);
  const unsigned prev = __ldg(slotPrev + s);
  if (h >= numCells || me >= n || prev >= n) return;  // unfilled slot (reported)
  const unsigned a = __ldg(off + h), b = __ldg(off + h + 1);
  unsigned dst = s;
  if (b - a <= kFixupMaxCell) {
    unsigned r = 0;
    for (unsigned t = a; t < b; ++t) r += __ldg(slotOrig + t) < me ? 1u : 0u;
    dst = a + r;
  } else if (s == a) {
    atomicOr(status, (unsigned)kStatusCellOverflow);
  }
  if (dst >= n) return;
  hashOut[dst] = h;
  indexOut[dst] = me;
  sortedPos[dst] = ldg4(prevPos + prev);
  sortedVel[dst] = ldg4(prevVel + prev);
}

// cellStart/cellEnd from the prefix table (cellEnd of empty cells untouched,
// as the reference leaves it).
__global__ void __launch_bounds__(256)
kCellTables(const unsigned *__restrict__ off, unsigned *__restrict__ cellStart,
            unsigned *__restrict__ cellEnd, unsigned numCells) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < numCells; c += stride) {
    unsigned a = __ldg(off + c), b = __ldg(off + c + 1);
    if (a < b) {
      cellStart[c] = a;
      cellEnd[c] = b;
    } else {
      cellStart[c] = kEmpty;
    }
  }
}

// First step of fcdemUpdate: integrate + calcHash + count.
__global__ void __launch_bounds__(256)
kIntegrateHashCount(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt,
                    unsigned *__restrict__ hash, unsigned *__restrict__ rank,
                    unsigned *__restrict__ cnt, unsigned n, KParams kp) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  float r = kp.radiusFromW ? p4.w : kp.p.particleRadius;
  integrateOne(p, v, dt, r, kp.p);
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, v4.w);
  int3 g = gridPos(p.x, p.y, p.z, kp.p);
  unsigned h = gridHash(g.x, g.y, g.z, kp.p);
  hash[i] = h;
  rank[i] = atomicAdd(cnt + h, 1u);
}

}  // namespace

// Buffers of the pipeline, kept in the context between calls: cnt (all zero
// between calls) and off over numCells + 1 cells, rank/slotKey/slotIdx over
// the particles, and the scan's look-back words.
static bool countBuffers(Context &c, unsigned n, unsigned numCells, CountBuffers &b) {
  const size_t m = (size_t)numCells + 1;
  const unsigned tiles = (unsigned)((m + kScanTile - 1) / kScanTile);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const size_t need = 2 * al(m * 4) + 4 * al((size_t)n * 4) + al((size_t)(tiles + 1) * 4);
  if (c.countBuf == nullptr || c.countBytes < need || c.countCells != numCells) {
    if (!cudaOk(cudaDeviceSynchronize())) return false;
    if (c.countBuf) cudaFree(c.countBuf);
    c.countBuf = nullptr;
    c.countBytes = 0;
    if (cudaMalloc(&c.countBuf, need) != cudaSuccess) {
      cudaGetLastError();
      c.countBuf = nullptr;
      setError(FCDEM_ERR_ALLOC);
      return false;
    }
    c.countBytes = need;
    c.countCells = numCells;
    if (!cudaOk(cudaMemset(c.countBuf, 0, need))) return false;  // cnt starts at zero
  }
  char *p = (char *)c.countBuf;
  b.cnt = (unsigned *)p;
  p += al(m * 4);
  b.off = (unsigned *)p;
  p += al(m * 4);
  b.rank = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotKey = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotIdx = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotPrev = (unsigned *)p;
  p += al((size_t)n * 4);
  b.lookback = (unsigned *)p;
  b.scanTiles = tiles;
  return true;
}

bool countPipelineBegin(Context &c, float4 *pos, float4 *vel, float dt, unsigned *hash,
                        unsigned n, unsigned numCells, const KParams &kp, CountBuffers &b) {
  if (!countBuffers(c, n, numCells, b)) return false;
  kIntegrateHashCount<<<(n + 255) / 256, 256, 0, curStream()>>>(pos, vel, dt, hash, b.rank,
                                                                b.cnt, n, kp);
  return launchOk();
}

// scan + scatter + fix-up/gather for one step (the counts are in place).
// hashN/rankN/origOf/prevPos/prevVel are indexed by the previous order's
// entries (origOf == nullptr: entry i is particle i, the first step).
bool countPipelineSort(Context &c, const CountBuffers &b, const unsigned *origOf,
                       const float4 *prevPos, const float4 *prevVel, unsigned *hash,
                       unsigned *index, float4 *sortedPos, float4 *sortedVel, unsigned n,
                       unsigned numCells) {
  cudaStream_t st = curStream();
  const unsigned m = numCells + 1;
  if (!cudaOk(cudaMemsetAsync(b.lookback, 0, (size_t)(b.scanTiles + 1) * 4, st))) return false;
  kScanCells<<<b.scanTiles, kScanThreads, 0, st>>>(b.cnt, b.off, m, b.lookback,
                                                   b.lookback + b.scanTiles, c.dStatus);
  if (!launchOk()) return false;
  // hash holds the new hashes in entry order until the fix-up overwrites it
  kScatterCells<<<(n + 255) / 256, 256, 0, st>>>(hash, b.rank, origOf, b.off, b.slotKey,
                                                  b.slotIdx, b.slotPrev, n, numCells,
                                                  c.dStatus);
  if (!launchOk()) return false;
  kFixupGather<<<(n + 255) / 256, 256, 0, st>>>(b.slotKey, b.slotIdx, b.slotPrev, b.off, hash,
                                                 index, sortedPos, sortedVel, prevPos, prevVel,
                                                 n, numCells, c.dStatus);
  return launchOk();
}

bool countPipelineTables(const CountBuffers &b, unsigned *cellStart, unsigned *cellEnd,
                         unsigned numCells) {
  unsigned blocks = (numCells + 255) / 256;
  if (blocks > 152u * 16u) blocks = 152u * 16u;
  kCellTables<<<blocks, 256, 0, curStream()>>>(b.off, cellStart, cellEnd, numCells);
  return launchOk();
}

}  // namespace fcdem
