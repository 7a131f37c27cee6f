// fcdem_count.cu -- the cell counting-sort pipeline of fcdemUpdate.
//
// The reference re-sorts all particles by cell hash every step
// (thrust::sort_by_key, particleSystem.cu:265-270) and then scatters the
// cell ranges (reorderDataAndFindCellStartD).  Inside fcdemUpdate the same
// result comes from a counting sort over the cells:
//
//   count   the kernel that computes a particle's cell hash h (the fused
//           collide+integrate of the previous step, or kIntegrateHashCount)
//           also takes r = atomicAdd(&cnt[h], 1) and counts h's 4096-cell
//           tile in tileCnt;
//   scan    kScanTiles (one CTA; above 8192 tiles kScanTileBlocks and
//           kAddTileBlocks) scans the tile counts, kScanCells scans
//           each tile's cells from its tile offset -- no inter-CTA waits; a
//           tile without particles writes its constant offsets and skips
//           reading cnt.  off = exclusive prefix sum of cnt over C + 1 cells,
//           cnt and tileCnt are cleared for the next step; off[c] .. off[c+1]
//           is cell c's range, empty or not;
//   scatter kScatterCells: slot off[h] + r receives (h, particle);
//   fix-up  kFixupGather: the atomic ranks order a cell's members
//           arbitrarily, so each slot re-ranks its particle among the
//           members of its cell by particle index (the order of the
//           reference's stable sort), then writes hash/index in sorted order
//           and gathers pos/vel into sortedPos/sortedVel (the reorder).
//
// The collide kernel reads `off` instead of cellStart/cellEnd.  At the end of
// fcdemUpdate kCellTables writes cellStart/cellEnd from `off`, so every array
// holds what the reference's stages leave.  A cell with more than
// kFixupMaxCell members is left out of the per-slot re-rank (its cost grows
// with the square of the cell) and listed instead; kFixupLarge then gives each
// listed cell one CTA that ranks its members by particle index, whatever the
// cell's size: with a bitmap of their indices when the indices are dense
// enough, else with a stable block radix sort.
#include "fcdem_dem.cuh"

namespace fcdem {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096 cells
constexpr int kTileShift = 12;  // log2(kScanTile)
constexpr unsigned kEmpty = 0xffffffffu;
static_assert((1 << kTileShift) == kScanTile, "tile shift");

// Exclusive prefix sums of the per-tile counts (one tile = kScanTile cells):
// tileOff[t] = sum of tileCnt[0..t), tileOff[tiles] = the total; tileCnt is
// cleared for the next step.  One CTA of 1024 threads, tiles in chunks.
__global__ void __launch_bounds__(1024)
kScanTiles(unsigned *__restrict__ tileCnt, unsigned *__restrict__ tileOff, unsigned tiles,
           unsigned *__restrict__ largeCount) {
  __shared__ unsigned sWarp[32];
  __shared__ unsigned sCarry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    sCarry = 0;
    *largeCount = 0u;  // the fix-up lists this step's large cells afresh
  }
  __syncthreads();
  for (unsigned base = 0; base < tiles; base += 1024) {
    const unsigned t = base + tid;
    const unsigned v = t < tiles ? tileCnt[t] : 0u;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sWarp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned w = sWarp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      sWarp[lane] = w;
    }
    __syncthreads();
    const unsigned carry = sCarry;
    if (t < tiles) {
      tileOff[t] = carry + (warp ? sWarp[warp - 1] : 0u) + x - v;
      tileCnt[t] = 0u;
    }
    __syncthreads();
    if (tid == 0) sCarry = carry + sWarp[31];
    __syncthreads();
  }
  if (tid == 0) tileOff[tiles] = sCarry;
}

// The same prefix over many tiles (batches of many scenes: tens of
// thousands of tiles), in two short launches instead of one CTA walking them
// all: kScanTileBlocks scans each block of 1024 tile counts and writes its
// total, kAddTileBlocks adds the totals of the blocks before.
constexpr unsigned kTileBlock = 1024;
constexpr unsigned kTilesOneCta = 8192;  // up to this many tiles kScanTiles runs alone

__global__ void __launch_bounds__(kTileBlock)
kScanTileBlocks(unsigned *__restrict__ tileCnt, unsigned *__restrict__ tileOff, unsigned tiles,
                unsigned *__restrict__ blockSum, unsigned *__restrict__ largeCount) {
  __shared__ unsigned sWarp[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (blockIdx.x == 0 && tid == 0) *largeCount = 0u;
  const unsigned t = blockIdx.x * kTileBlock + tid;
  const unsigned v = t < tiles ? tileCnt[t] : 0u;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sWarp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned w = sWarp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sWarp[lane] = w;
  }
  __syncthreads();
  if (t < tiles) {
    tileOff[t] = (warp ? sWarp[warp - 1] : 0u) + x - v;
    tileCnt[t] = 0u;
  }
  if (tid == 0) blockSum[blockIdx.x] = sWarp[31];
}

__global__ void __launch_bounds__(kTileBlock)
kAddTileBlocks(unsigned *__restrict__ tileOff, unsigned tiles,
               const unsigned *__restrict__ blockSum) {
  __shared__ unsigned sPart[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned part = 0;
  for (unsigned b = tid; b < blockIdx.x; b += kTileBlock) part += __ldg(blockSum + b);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) sPart[warp] = part;
  __syncthreads();
  unsigned carry = 0;
  for (int w = 0; w < (int)(kTileBlock / 32); ++w) carry += sPart[w];
  const unsigned t = blockIdx.x * kTileBlock + tid;
  if (t < tiles) tileOff[t] += carry;
  if (blockIdx.x == gridDim.x - 1 && tid == 0)
    tileOff[tiles] = carry + __ldg(blockSum + blockIdx.x);
}

// off[c] = tileOff[tile] + exclusive prefix of cnt within the tile, cnt
// cleared.  A tile without particles only writes its constant offsets, and
// not even those when off already holds them: tileOffPrev[tile] records the
// constant a tile's offsets were last written with (0xffffffff after a tile
// with particles, whose offsets vary), so a tile that stays empty with the
// same prefix -- the common case in sparse grids: the cells above and below
// a pile -- is left as it is.
// Round q of a tile covers cells q*1024 .. +1024, thread t the four at 4t
// (16-byte accesses, coalesced).
__global__ void __launch_bounds__(kScanThreads)
kScanCells(unsigned *__restrict__ cnt, unsigned *__restrict__ off, unsigned m,
           const unsigned *__restrict__ tileOff, unsigned *__restrict__ tileOffPrev) {
  __shared__ unsigned sWarp[kScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned tile = blockIdx.x;
  constexpr int kRounds = kScanItems / 4;
  const size_t tbase = (size_t)tile * kScanTile;
  const unsigned t0 = __ldg(tileOff + tile), t1 = __ldg(tileOff + tile + 1);
  const unsigned prev = tileOffPrev[tile];  // read by every thread before thread 0 writes
  if (t0 == t1) {  // empty tile: every cell starts (and ends) at t0
    if (prev == t0) return;  // off already holds t0 in every cell of the tile
    __syncthreads();
    if (tid == 0) tileOffPrev[tile] = t0;
#pragma unroll
    for (int q = 0; q < kRounds; ++q) {
      const size_t c0 = tbase + (size_t)q * (kScanThreads * 4) + (size_t)tid * 4;
      if (c0 + 4 <= m) {
        reinterpret_cast<uint4 *>(off + c0)[0] = make_uint4(t0, t0, t0, t0);
      } else {
        for (int k = 0; k < 4; ++k)
          if (c0 + k < m) off[c0 + k] = t0;
      }
    }
    return;
  }
  __syncthreads();
  if (tid == 0 && prev != 0xffffffffu) tileOffPrev[tile] = 0xffffffffu;  // offsets vary
  uint4 v[kRounds];
  unsigned excl[kRounds];
#pragma unroll
  for (int q = 0; q < kRounds; ++q) {  // all loads in flight before the scans
    const size_t c0 = tbase + (size_t)q * (kScanThreads * 4) + (size_t)tid * 4;
    if (c0 + 4 <= m) {
      v[q] = reinterpret_cast<const uint4 *>(cnt + c0)[0];
    } else {
      v[q].x = c0 < m ? cnt[c0] : 0u;
      v[q].y = c0 + 1 < m ? cnt[c0 + 1] : 0u;
      v[q].z = c0 + 2 < m ? cnt[c0 + 2] : 0u;
      v[q].w = c0 + 3 < m ? cnt[c0 + 3] : 0u;
    }
  }
  unsigned carry = 0;
#pragma unroll
  for (int q = 0; q < kRounds; ++q) {
    const unsigned sum = v[q].x + v[q].y + v[q].z + v[q].w;
    unsigned x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sWarp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned w = lane < kScanThreads / 32 ? sWarp[lane] : 0u;
#pragma unroll
      for (int o = 1; o < kScanThreads / 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      if (lane < kScanThreads / 32) sWarp[lane] = w;
    }
    __syncthreads();
    excl[q] = carry + (warp ? sWarp[warp - 1] : 0u) + x - sum;
    carry += sWarp[kScanThreads / 32 - 1];
    __syncthreads();  // sWarp is reused by the next round
  }
#pragma unroll
  for (int q = 0; q < kRounds; ++q) {
    const size_t c0 = tbase + (size_t)q * (kScanThreads * 4) + (size_t)tid * 4;
    uint4 o;
    o.x = t0 + excl[q];
    o.y = o.x + v[q].x;
    o.z = o.y + v[q].y;
    o.w = o.z + v[q].z;
    if (c0 + 4 <= m) {
      reinterpret_cast<uint4 *>(off + c0)[0] = o;
      reinterpret_cast<uint4 *>(cnt + c0)[0] = make_uint4(0u, 0u, 0u, 0u);
    } else {
      const unsigned ov[4] = {o.x, o.y, o.z, o.w};
      for (int k = 0; k < 4; ++k)
        if (c0 + k < m) {
          off[c0 + k] = ov[k];
          cnt[c0 + k] = 0u;
        }
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

// Largest cell that the per-slot re-rank handles (each slot reads every
// member of its cell).
constexpr unsigned kFixupMaxCell = 1024;

// Capacity of the large-cell list: a listed cell has more than kFixupMaxCell
// of the n particles, so at most n / (kFixupMaxCell + 1) cells are listed.
inline unsigned largeCapacity(unsigned n) { return n / (kFixupMaxCell + 1) + 1; }

// Stable order inside each cell + the reorder gather.  The particle of slot
// s is re-ranked among its cell's members by particle index; its position and
// velocity are gathered from entry slotPrev[s] of the previous order.  A cell
// above kFixupMaxCell members is appended to large[1..] (large[0] counts) by
// its first slot and left to kFixupLarge.
__global__ void __launch_bounds__(256)
kFixupGather(const unsigned *__restrict__ slotKey, const unsigned *__restrict__ slotOrig,
             const unsigned *__restrict__ slotPrev, const unsigned *__restrict__ off,
             unsigned *__restrict__ hashOut, unsigned *__restrict__ indexOut,
             float4 *__restrict__ sortedPos, float4 *__restrict__ sortedVel,
             const float4 *__restrict__ prevPos, const float4 *__restrict__ prevVel,
             unsigned n, unsigned numCells, unsigned *__restrict__ large, unsigned largeCap,
             unsigned *status) {
  unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const unsigned h = __ldg(slotKey + s);
  const unsigned me = __ldg(slotOrig + s);
  const unsigned prev = __ldg(slotPrev + s);
  if (h >= numCells || me >= n || prev >= n) return;  // unfilled slot (reported)
  const unsigned a = __ldg(off + h), b = __ldg(off + h + 1);
  if (b - a > kFixupMaxCell) {
    if (s == a) {
      const unsigned k = atomicAdd(large, 1u);
      if (k < largeCap)
        large[1 + k] = h;
      else
        atomicOr(status, (unsigned)kStatusCellOverflow);
    }
    return;
  }
  unsigned r = 0;
  for (unsigned t = a; t < b; ++t) r += __ldg(slotOrig + t) < me ? 1u : 0u;
  const unsigned dst = a + r;
  if (dst >= n) return;
  hashOut[dst] = h;
  indexOut[dst] = me;
  sortedPos[dst] = ldg4(prevPos + prev);
  sortedVel[dst] = ldg4(prevVel + prev);
}

constexpr int kLargeThreads = 1024;
constexpr int kLargeWarps = kLargeThreads / 32;
constexpr int kBitmapSlots = 16;  // CTAs of kFixupLarge that own a bitmap

// Words of one bitmap slot: a presence bit per particle index.
__host__ __device__ inline size_t bitmapWords(unsigned n) { return (size_t)n / 32 + 1; }

struct LargeSmem {
  unsigned bin[256];                  // running base of each digit
  unsigned total[256];                // a chunk's count of each digit
  unsigned part[8];                   // warp totals of the digit scan
  unsigned warpCnt[kLargeWarps][256]; // per-warp digit counts of a chunk
  unsigned warpSum[kLargeWarps];      // bitmap path: popcount of each warp's run
  unsigned lo, hi;                    // bitmap path: smallest / largest member index
};

// Bitmap rank of a large cell's members (the members' particle indices are
// distinct): bit i of `bits` is set for member index i; pre[w] is the number
// of set bits in words w0 .. w-1; the rank of member i among the cell's
// members is pre[i / 32] + the set bits below i in its word.  Words w0..w1
// (the members' index span) are cleared, filled, counted and scanned: the
// work grows with the span, not with the member count, so the caller takes
// this path when the span is at most kBitmapSpan words per member.
constexpr unsigned kBitmapSpan = 16;

__device__ void bitmapRanks(const unsigned *slotOrig, unsigned a, unsigned c, unsigned n,
                            unsigned w0, unsigned w1, unsigned *bits, unsigned *pre,
                            LargeSmem &sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (unsigned w = w0 + tid; w <= w1; w += kLargeThreads) bits[w] = 0u;
  __syncthreads();
  for (unsigned t = tid; t < c; t += kLargeThreads) {
    const unsigned me = slotOrig[a + t];
    if (me < n) atomicOr(bits + (me >> 5), 1u << (me & 31u));
  }
  __syncthreads();
  // each warp owns a contiguous run of words: its total, then the scan
  const unsigned span = w1 - w0 + 1u;
  const unsigned run = ((span + kLargeWarps - 1u) / kLargeWarps + 31u) & ~31u;
  const unsigned ws = w0 + (unsigned)warp * run;
  const unsigned we = min(ws + run, w1 + 1u);
  unsigned sum = 0;
  for (unsigned w = ws + lane; w < we; w += 32) sum += __popc(bits[w]);
  sum = __reduce_add_sync(0xffffffffu, sum);
  if (lane == 0) sm.warpSum[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    const unsigned v = sm.warpSum[lane];
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    sm.warpSum[lane] = x - v;
  }
  __syncthreads();
  unsigned carry = sm.warpSum[warp];
  for (unsigned base = ws; base < we; base += 32) {
    const unsigned w = base + lane;
    const unsigned v = w < we ? __popc(bits[w]) : 0u;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (w < we) pre[w] = carry + x - v;
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
  __syncthreads();
}

// One stable pass of a block-wide LSD radix sort: src[0..c) -> dst[0..c)
// by the 8-bit digit at bit `shift`.  Chunks of kLargeThreads entries go in
// order; inside a chunk an entry's place is its digit's running base + the
// count of that digit in earlier warps + its rank among its warp's peers.
__device__ void largeRadixPass(const unsigned long long *src, unsigned long long *dst,
                               unsigned c, int shift, LargeSmem &sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 256) sm.bin[tid] = 0u;
  __syncthreads();
  for (unsigned t = tid; t < c; t += kLargeThreads)
    atomicAdd(&sm.bin[(unsigned)(src[t] >> shift) & 255u], 1u);
  __syncthreads();
  unsigned v = 0, x = 0;
  if (tid < 256) {  // exclusive scan of the 256 digit counts, warps 0..7
    v = sm.bin[tid];
    x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sm.part[warp] = x;
  }
  __syncthreads();
  if (tid < 256) {
    unsigned before = 0;
    for (int w = 0; w < warp; ++w) before += sm.part[w];
    sm.bin[tid] = before + x - v;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (unsigned base = 0; base < c; base += kLargeThreads) {
    for (int q = tid; q < kLargeWarps * 256; q += kLargeThreads) (&sm.warpCnt[0][0])[q] = 0u;
    __syncthreads();
    const unsigned t = base + tid;
    const bool valid = t < c;
    const unsigned long long e = valid ? src[t] : 0ull;
    const unsigned d = valid ? ((unsigned)(e >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lt);
    if (valid && rank == 0) sm.warpCnt[warp][d] = __popc(peers);
    __syncthreads();
    if (tid < 256) {  // per digit: exclusive prefix over the warps
      unsigned run = 0;
      for (int w = 0; w < kLargeWarps; ++w) {
        const unsigned k = sm.warpCnt[w][tid];
        sm.warpCnt[w][tid] = run;
        run += k;
      }
      sm.total[tid] = run;
    }
    __syncthreads();
    if (valid) dst[sm.bin[d] + sm.warpCnt[warp][d] + rank] = e;
    __syncthreads();
    if (tid < 256) sm.bin[tid] += sm.total[tid];
    __syncthreads();
  }
}

// The large cells listed by kFixupGather, one CTA per cell at a time.  A
// CTA with a bitmap slot (blockIdx < kBitmapSlots) ranks a cell whose
// members' index span is at most kBitmapSpan words per member with
// bitmapRanks and gathers each member straight to its ranked place.
// Otherwise the members (particle index, previous entry) are sorted by
// particle index in the cell's own range of sortedPos (16 bytes per member:
// two 8-byte arrays of the cell's size), written back to slotOrig/slotPrev,
// then gathered as in kFixupGather.  idBits = bits of the largest particle
// index; bitmaps = kBitmapSlots slots of 2 * bitmapWords(n) words (the bits,
// then the word prefix), or nullptr for the sort only.
__global__ void __launch_bounds__(kLargeThreads)
kFixupLarge(unsigned *__restrict__ slotOrig, unsigned *__restrict__ slotPrev,
            const unsigned *__restrict__ off, const unsigned *__restrict__ large,
            unsigned largeCap, unsigned *__restrict__ hashOut, unsigned *__restrict__ indexOut,
            float4 *__restrict__ sortedPos, float4 *__restrict__ sortedVel,
            const float4 *__restrict__ prevPos, const float4 *__restrict__ prevVel, unsigned n,
            int idBits, unsigned *__restrict__ bitmaps) {
  __shared__ LargeSmem sm;
  const unsigned count = min(large[0], largeCap);
  const int tid = threadIdx.x;
  const size_t words = bitmapWords(n);
  unsigned *bits = blockIdx.x < (unsigned)kBitmapSlots && bitmaps
                       ? bitmaps + (size_t)blockIdx.x * 2u * words
                       : nullptr;
  for (unsigned k = blockIdx.x; k < count; k += gridDim.x) {
    const unsigned h = large[1 + k];
    const unsigned a = off[h], b = off[h + 1];
    if (b > n || a >= b) continue;  // cannot happen for a listed cell
    const unsigned c = b - a;
    if (bits) {
      // the members' index span decides between the bitmap and the sort
      if (tid == 0) {
        sm.lo = 0xffffffffu;
        sm.hi = 0u;
      }
      __syncthreads();
      unsigned lo = 0xffffffffu, hi = 0u;
      for (unsigned t = tid; t < c; t += kLargeThreads) {
        const unsigned me = slotOrig[a + t];
        if (me < n) {
          lo = min(lo, me);
          hi = max(hi, me);
        }
      }
      lo = __reduce_min_sync(0xffffffffu, lo);
      hi = __reduce_max_sync(0xffffffffu, hi);
      if ((tid & 31) == 0) {
        atomicMin(&sm.lo, lo);
        atomicMax(&sm.hi, hi);
      }
      __syncthreads();
      const unsigned mlo = sm.lo, mhi = sm.hi;
      const unsigned w0 = mlo >> 5, w1 = mhi >> 5;
      if (mlo <= mhi && w1 - w0 + 1u <= kBitmapSpan * c) {
        unsigned *pre = bits + words;
        bitmapRanks(slotOrig, a, c, n, w0, w1, bits, pre, sm);
        for (unsigned t = tid; t < c; t += kLargeThreads) {
          const unsigned me = slotOrig[a + t], prev = slotPrev[a + t];
          if (me >= n || prev >= n) continue;  // unfilled slot (reported by the scatter)
          const unsigned wd = me >> 5;
          const unsigned dst = a + pre[wd] + __popc(bits[wd] & ((1u << (me & 31u)) - 1u));
          hashOut[dst] = h;
          indexOut[dst] = me;
          sortedPos[dst] = ldg4(prevPos + prev);
          sortedVel[dst] = ldg4(prevVel + prev);
        }
        __syncthreads();  // the bitmap is reused by the next cell
        continue;
      }
    }
    unsigned long long *A = reinterpret_cast<unsigned long long *>(sortedPos + a);
    unsigned long long *B = A + c;
    for (unsigned t = tid; t < c; t += kLargeThreads)
      A[t] = ((unsigned long long)slotOrig[a + t] << 32) | slotPrev[a + t];
    __syncthreads();
    for (int shift = 0; shift < idBits; shift += 8) {
      largeRadixPass(A, B, c, 32 + shift, sm);
      unsigned long long *tmp = A;
      A = B;
      B = tmp;
    }
    for (unsigned t = tid; t < c; t += kLargeThreads) {
      const unsigned long long e = A[t];
      slotOrig[a + t] = (unsigned)(e >> 32);
      slotPrev[a + t] = (unsigned)e;
    }
    __syncthreads();
    for (unsigned t = tid; t < c; t += kLargeThreads) {
      const unsigned me = slotOrig[a + t], prev = slotPrev[a + t];
      if (me >= n || prev >= n) continue;  // unfilled slot (reported by the scatter)
      hashOut[a + t] = h;
      indexOut[a + t] = me;
      sortedPos[a + t] = ldg4(prevPos + prev);
      sortedVel[a + t] = ldg4(prevVel + prev);
    }
    __syncthreads();
  }
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

// First step of fcdemUpdate: integrate + calcHash + count (the tile counts
// follow in kTileReduce).
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

// tileCnt[t] = sum of cnt over tile t (after kIntegrateHashCount, whose
// particle-order cells are scattered over the tiles: summing the counts once
// is cheaper than one atomic per particle on the few tile counters).
__global__ void __launch_bounds__(kScanThreads)
kTileReduce(const unsigned *__restrict__ cnt, unsigned *__restrict__ tileCnt, unsigned m) {
  __shared__ unsigned sWarp[kScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t tbase = (size_t)blockIdx.x * kScanTile;
  unsigned sum = 0;
#pragma unroll
  for (int q = 0; q < kScanItems / 4; ++q) {
    const size_t c0 = tbase + (size_t)q * (kScanThreads * 4) + (size_t)tid * 4;
    if (c0 + 4 <= m) {
      uint4 v = reinterpret_cast<const uint4 *>(cnt + c0)[0];
      sum += v.x + v.y + v.z + v.w;
    } else {
      for (int k = 0; k < 4; ++k)
        if (c0 + k < m) sum += cnt[c0 + k];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) sWarp[warp] = sum;
  __syncthreads();
  if (tid == 0) {
    unsigned t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += sWarp[w];
    tileCnt[blockIdx.x] = t;
  }
}

}  // namespace

// First step of a batch: scene of particle i from sceneOf, integrate in the
// scene's box, global cell id = the scene's cellBase + local hash.
template <bool kRadiusFromW>
__global__ void __launch_bounds__(256)
kBatchIntegrateHashCount(const BatchScene *__restrict__ scenes,
                         const unsigned *__restrict__ sceneOf, float4 *__restrict__ pos,
                         float4 *__restrict__ vel, float dt, unsigned *__restrict__ hash,
                         unsigned *__restrict__ rank, unsigned *__restrict__ cnt, unsigned n) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BatchScene &S = scenes[__ldg(sceneOf + i)];
  const SimParams &P = S.p;
  float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  float r = kRadiusFromW ? p4.w : P.particleRadius;
  integrateOneBox(p, v, dt, r, P, S.lo, S.hi);
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, v4.w);
  int3 g = gridPos(p.x, p.y, p.z, P);
  unsigned h = S.cellBase + gridHash(g.x, g.y, g.z, P);
  hash[i] = h;
  rank[i] = atomicAdd(cnt + h, 1u);
}

// Buffers of the pipeline, kept in the context between calls: cnt (all zero
// between calls) and off over numCells + 1 cells, rank/slotKey/slotIdx over
// the particles, and the scan's look-back words.
static bool countBuffers(Context &c, unsigned n, unsigned numCells, CountBuffers &b) {
  return countBuffersIn(c.countBuf, c.countBytes, c.countCells, n, numCells, b);
}

bool countBuffersIn(void *&buf, size_t &bytes, unsigned &cells, unsigned n, unsigned numCells,
                    CountBuffers &b) {
  const size_t m = (size_t)numCells + 1;
  const unsigned tiles = (unsigned)((m + kScanTile - 1) / kScanTile);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const unsigned largeCap = largeCapacity(n);
  const unsigned tileBlocks = (tiles + kTileBlock - 1) / kTileBlock;
  const size_t need = 2 * al(m * 4) + 4 * al((size_t)n * 4) + 3 * al((size_t)(tiles + 1) * 4) +
                      al(((size_t)largeCap + 1) * 4) + al((size_t)tileBlocks * 4) +
                      al((size_t)kBitmapSlots * 2 * bitmapWords(n) * 4);
  if (buf == nullptr || bytes < need || cells != numCells) {
    if (!cudaOk(cudaDeviceSynchronize())) return false;
    if (buf) cudaFree(buf);
    buf = nullptr;
    bytes = 0;
    if (cudaMalloc(&buf, need) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      setError(FCDEM_ERR_ALLOC);
      return false;
    }
    bytes = need;
    cells = numCells;
    if (!cudaOk(cudaMemset(buf, 0, need))) return false;  // cnt starts at zero
    // no tile's offsets are known yet (see kScanCells)
    const size_t prevAt = 2 * al(m * 4) + 2 * al((size_t)(tiles + 1) * 4);
    if (!cudaOk(cudaMemset((char *)buf + prevAt, 0xff, (size_t)(tiles + 1) * 4))) return false;
  }
  // The arrays that must stay zero between calls (cnt, tileCnt) sit first,
  // at offsets that depend on the cell count only, so that a call with
  // another particle count reuses them in place.
  char *p = (char *)buf;
  b.cnt = (unsigned *)p;
  p += al(m * 4);
  b.tileCnt = (unsigned *)p;
  p += al((size_t)(tiles + 1) * 4);
  b.off = (unsigned *)p;
  p += al(m * 4);
  b.tileOff = (unsigned *)p;
  p += al((size_t)(tiles + 1) * 4);
  b.tileOffPrev = (unsigned *)p;
  p += al((size_t)(tiles + 1) * 4);
  b.rank = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotKey = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotIdx = (unsigned *)p;
  p += al((size_t)n * 4);
  b.slotPrev = (unsigned *)p;
  p += al((size_t)n * 4);
  b.large = (unsigned *)p;
  b.largeCap = largeCap;
  p += al(((size_t)largeCap + 1) * 4);
  b.tileBlockSum = (unsigned *)p;
  p += al((size_t)tileBlocks * 4);
  b.bitmaps = (unsigned *)p;  // cleared where used (kFixupLarge)
  b.scanTiles = tiles;
  return true;
}

bool countPipelineBegin(Context &c, float4 *pos, float4 *vel, float dt, unsigned *hash,
                        unsigned n, unsigned numCells, const KParams &kp, CountBuffers &b) {
  if (!countBuffers(c, n, numCells, b)) return false;
  kIntegrateHashCount<<<(n + 255) / 256, 256, 0, curStream()>>>(pos, vel, dt, hash, b.rank,
                                                                b.cnt, n, kp);
  if (!launchOk()) return false;
  kTileReduce<<<b.scanTiles, kScanThreads, 0, curStream()>>>(b.cnt, b.tileCnt, numCells + 1);
  return launchOk();
}

bool countPipelineBeginBatch(const BatchScene *scenes, const unsigned *sceneOf, bool radiusFromW,
                             float4 *pos, float4 *vel, float dt, unsigned *hash, unsigned n,
                             unsigned numCells, const CountBuffers &b) {
  if (radiusFromW)
    kBatchIntegrateHashCount<true><<<(n + 255) / 256, 256, 0, curStream()>>>(
        scenes, sceneOf, pos, vel, dt, hash, b.rank, b.cnt, n);
  else
    kBatchIntegrateHashCount<false><<<(n + 255) / 256, 256, 0, curStream()>>>(
        scenes, sceneOf, pos, vel, dt, hash, b.rank, b.cnt, n);
  if (!launchOk()) return false;
  kTileReduce<<<b.scanTiles, kScanThreads, 0, curStream()>>>(b.cnt, b.tileCnt, numCells + 1);
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
  if (b.scanTiles <= kTilesOneCta) {
    kScanTiles<<<1, 1024, 0, st>>>(b.tileCnt, b.tileOff, b.scanTiles, b.large);
    if (!launchOk()) return false;
  } else {
    const unsigned blocks = (b.scanTiles + kTileBlock - 1) / kTileBlock;
    kScanTileBlocks<<<blocks, kTileBlock, 0, st>>>(b.tileCnt, b.tileOff, b.scanTiles,
                                                   b.tileBlockSum, b.large);
    if (!launchOk()) return false;
    kAddTileBlocks<<<blocks, kTileBlock, 0, st>>>(b.tileOff, b.scanTiles, b.tileBlockSum);
    if (!launchOk()) return false;
  }
  kScanCells<<<b.scanTiles, kScanThreads, 0, st>>>(b.cnt, b.off, m, b.tileOff,
                                                    b.tileOffPrev);
  if (!launchOk()) return false;
  // hash holds the new hashes in entry order until the fix-up overwrites it
  kScatterCells<<<(n + 255) / 256, 256, 0, st>>>(hash, b.rank, origOf, b.off, b.slotKey,
                                                  b.slotIdx, b.slotPrev, n, numCells,
                                                  c.dStatus);
  if (!launchOk()) return false;
  kFixupGather<<<(n + 255) / 256, 256, 0, st>>>(b.slotKey, b.slotIdx, b.slotPrev, b.off, hash,
                                                 index, sortedPos, sortedVel, prevPos, prevVel,
                                                 n, numCells, b.large, b.largeCap, c.dStatus);
  if (!launchOk()) return false;
  // Returns at once when the fix-up listed no cell (the common case).
  const unsigned largeCtas = b.largeCap < numSms() ? b.largeCap : numSms();  // one per SM at most
  kFixupLarge<<<largeCtas, kLargeThreads, 0, st>>>(b.slotIdx, b.slotPrev, b.off, b.large,
                                                   b.largeCap, hash, index, sortedPos,
                                                   sortedVel, prevPos, prevVel, n, keyBits(n),
                                                   b.bitmaps);
  return launchOk();
}

bool countPipelineTables(const CountBuffers &b, unsigned *cellStart, unsigned *cellEnd,
                         unsigned numCells) {
  unsigned blocks = (numCells + 255) / 256;
  if (blocks > numSms() * 16u) blocks = numSms() * 16u;
  kCellTables<<<blocks, 256, 0, curStream()>>>(b.off, cellStart, cellEnd, numCells);
  return launchOk();
}

}  // namespace fcdem
