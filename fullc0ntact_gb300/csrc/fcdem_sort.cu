// fcdem_sort.cu -- stable LSD radix sort of (key, value) pairs: the stage
// the reference hands to thrust::sort_by_key (particleSystem.cu:265-270).
//
// One upsweep kernel builds the digit histograms of every pass in one read of
// the keys; then each pass is a single "onesweep" kernel: a CTA takes the
// next tile (4096 keys) from an atomic counter, ranks its keys stably by
// digit with warp ballots, publishes its per-digit counts, resolves its
// global offsets by decoupled look-back over the tiles before it (each digit's
// thread reads kLookWindow predecessors per round), stages the tile in shared
// memory in digit order and writes it out in runs.
//
// Every look-back wait is bounded: after a limit of rounds (kSortWaitRounds,
// settable with fcdemSetSortWaitLimit) the CTA records kStatusTimeout in the
// device status word and carries on with the part of its prefix it has
// summed, so a fault in the protocol turns into an error the host reads,
// never into a hung GPU.  Such a partial prefix is at most the true one, so
// every write of the pass still lands inside [0, n) (the write-out also
// guards it): the result is wrong, the memory outside the arrays untouched.
#include <atomic>
#include <mutex>

#include "fcdem_internal.cuh"

namespace fcdem {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kThreads = 256;  // upsweep, and the fixed configuration
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096 keys (fixed configuration)
constexpr int kMaxPasses = 4;
constexpr unsigned kFlagAgg = 1u << 30;
constexpr unsigned kFlagPrefix = 2u << 30;
constexpr unsigned kValueMask = (1u << 30) - 1u;
constexpr unsigned kSortWaitRounds = 1u << 22;
constexpr int kLookWindow = 8;  // look-back tiles read per round

std::atomic<unsigned> g_sortWaitRounds{kSortWaitRounds};  // fcdemSetSortWaitLimit


__device__ __forceinline__ unsigned lanemaskLt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Mask of the lanes of `active` whose digit equals this lane's (8 ballots).
__device__ __forceinline__ unsigned digitPeers(unsigned d, unsigned active) {
  unsigned peers = active;
#pragma unroll
  for (int b = 0; b < kRadixBits; ++b) {
    unsigned bit = (d >> b) & 1u;
    unsigned vote = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? vote : ~vote;
  }
  return peers;
}

__device__ __forceinline__ unsigned ldVolatile(const unsigned *p) {
  return *(const volatile unsigned *)p;
}
__device__ __forceinline__ void stVolatile(unsigned *p, unsigned v) {
  *(volatile unsigned *)p = v;
}

// Exclusive scan of one value per thread over a block of THREADS threads.
template <int THREADS>
__device__ __forceinline__ unsigned blockExclusiveScan(unsigned v, unsigned *warpSums) {
  constexpr int kWarps = THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warpSums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned s = lane < kWarps ? warpSums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kWarps) warpSums[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  unsigned before = warp ? warpSums[warp - 1] : 0u;
  unsigned r = before + x - v;
  __syncthreads();  // warpSums may be reused by the caller
  return r;
}

// Histograms of all `passes` digits; checks that no key has bits at or above
// `bits`.  hist must be zero on entry.  Each warp counts into its own copy
// of the histograms (shared-memory atomics of one warp only contend with its
// own lanes); a digit that all lanes of the warp share (sorted or clustered
// keys) is added once.  The copies are summed at the end.
constexpr int kUpWarps = kThreads / 32;
constexpr int kUpKeys = 4;
__global__ void __launch_bounds__(kThreads)
kUpsweep(const unsigned *__restrict__ keys, unsigned n, int passes, int bits,
         unsigned *__restrict__ hist, unsigned *__restrict__ status) {
  __shared__ unsigned sh[kUpWarps][kMaxPasses][kRadix];
  for (int k = threadIdx.x; k < kUpWarps * kMaxPasses * kRadix; k += kThreads)
    (&sh[0][0][0])[k] = 0;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bool bad = false;
  // kUpKeys keys per thread and round, their loads issued together
  const unsigned stride = gridDim.x * kThreads;
  const unsigned nRound = (n + 31u) & ~31u;
  for (unsigned i0 = blockIdx.x * kThreads + threadIdx.x; i0 < nRound; i0 += kUpKeys * stride) {
    unsigned k[kUpKeys];
    bool valid[kUpKeys];
#pragma unroll
    for (int u = 0; u < kUpKeys; ++u) {
      const unsigned i = i0 + u * stride;
      valid[u] = i < n;
      k[u] = valid[u] ? __ldg(keys + i) : 0u;
    }
#pragma unroll
    for (int u = 0; u < kUpKeys; ++u) {
      if (i0 + u * stride >= nRound) break;  // warp-uniform: nRound and stride are multiples of 32
      if (valid[u] && bits < 32 && (k[u] >> bits) != 0u) bad = true;
      const unsigned active = __ballot_sync(0xffffffffu, valid[u]);
      for (int p = 0; p < passes; ++p) {
        const unsigned d = (k[u] >> (p * kRadixBits)) & (kRadix - 1);
        int same = 0;
        __match_all_sync(0xffffffffu, valid[u] ? d : kRadix, &same);
        if (same) {
          if (lane == 0 && active) atomicAdd(&sh[warp][p][d], (unsigned)__popc(active));
        } else if (valid[u]) {
          atomicAdd(&sh[warp][p][d], 1u);
        }
      }
    }
  }
  if (bad) atomicOr(status, (unsigned)kStatusKeyRange);
  __syncthreads();
  for (int e = threadIdx.x; e < passes * kRadix; e += kThreads) {
    unsigned c = 0;
#pragma unroll
    for (int w = 0; w < kUpWarps; ++w) c += (&sh[w][0][0])[e];
    if (c) atomicAdd(hist + e, c);
  }
}

// One counting pass over digit `shift`, THREADS threads of ITEMS keys each
// (a tile of THREADS * ITEMS keys).  Threads 0..255 own one digit each in the
// count, look-back and scan phases.  lookback has one kRadix-word row per
// tile and must be zero on entry, as must *tileCounter.  valsIn == nullptr
// stands for the identity values 0, 1, ..., n-1.  Dynamic shared memory:
// onesweepSmem<THREADS, ITEMS>() bytes.
template <int THREADS, int ITEMS>
constexpr size_t onesweepSmem() {
  return (size_t)(THREADS / 32) * kRadix * 4 + 2 * kRadix * 4 + 32 * 4 + 16 +
         (size_t)2 * THREADS * ITEMS * 4;
}

template <int THREADS, int ITEMS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
kOnesweep(const unsigned *__restrict__ keysIn, const unsigned *__restrict__ valsIn,
          unsigned *__restrict__ keysOut, unsigned *__restrict__ valsOut,
          unsigned n, int shift, const unsigned *__restrict__ hist,
          unsigned *lookback, unsigned *tileCounter, unsigned *status, unsigned waitRounds) {
  static_assert(THREADS >= kRadix, "one thread per digit in the scan phases");
  constexpr int kWarps = THREADS / 32;
  constexpr int kTileKeys = THREADS * ITEMS;
  constexpr int kWarpKeys = 32 * ITEMS;
  extern __shared__ __align__(16) unsigned char smemRaw[];
  unsigned(*sWarpHist)[kRadix] = reinterpret_cast<unsigned(*)[kRadix]>(smemRaw);
  unsigned *sBinExcl = reinterpret_cast<unsigned *>(smemRaw + kWarps * kRadix * 4);
  int *sBase = reinterpret_cast<int *>(sBinExcl + kRadix);
  unsigned *sWarpSums = reinterpret_cast<unsigned *>(sBase + kRadix);
  unsigned *sTileP = sWarpSums + 32;
  unsigned *sKeys = sTileP + 4;
  unsigned *sVals = sKeys + kTileKeys;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) *sTileP = atomicAdd(tileCounter, 1u);
  for (int k = tid; k < kWarps * kRadix; k += THREADS) (&sWarpHist[0][0])[k] = 0;
  __syncthreads();
  const unsigned tile = *sTileP;
  const unsigned base = tile * (unsigned)kTileKeys;
  const unsigned wbase = base + warp * kWarpKeys;

  unsigned key[ITEMS], val[ITEMS], rank[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    unsigned idx = wbase + r * 32 + lane;
    bool valid = idx < n;
    key[r] = valid ? __ldg(keysIn + idx) : 0u;
    val[r] = valid ? (valsIn ? __ldg(valsIn + idx) : idx) : 0u;
  }

  // Stable rank inside the warp: rounds in position order, lanes in position
  // order within a round.
  const unsigned lt = lanemaskLt();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    unsigned idx = wbase + r * 32 + lane;
    bool valid = idx < n;
    unsigned active = __ballot_sync(0xffffffffu, valid);
    unsigned d = (key[r] >> shift) & (kRadix - 1);
    unsigned peers = digitPeers(d, active);
    unsigned before = valid ? sWarpHist[warp][d] : 0u;
    __syncwarp();
    if (valid && (peers & lt) == 0u) sWarpHist[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + __popc(peers & lt);
  }
  __syncthreads();

  // Thread b < 256 owns digit b: per-warp exclusive offsets, the tile count
  // and the decoupled look-back over the tiles before this one.
  const unsigned b = tid;
  const bool owner = tid < kRadix;
  unsigned count = 0, excl = 0;
  if (owner) {
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      unsigned c = sWarpHist[w][b];
      sWarpHist[w][b] = count;
      count += c;
    }
    unsigned *row = lookback + (size_t)tile * kRadix;
    if (tile == 0) {
      stVolatile(row + b, kFlagPrefix | count);
    } else {
      stVolatile(row + b, kFlagAgg | count);
      // Look back kLookWindow tiles per round: their words are loaded
      // together (one latency for the window) and consumed nearest first,
      // adding aggregates until an inclusive prefix; a tile that has not
      // published yet ends the round, and the next round starts there.  At
      // most waitRounds rounds: then the wait has run out (kStatusTimeout)
      // and excl keeps the aggregates summed so far.
      int t = (int)tile - 1;
      unsigned empty = 0;
      bool done = false;
      for (unsigned round = 0; !done; ++round) {
        if (round >= waitRounds) {
          atomicOr(status, (unsigned)kStatusTimeout);
          break;
        }
        unsigned w[kLookWindow];
#pragma unroll
        for (int j = 0; j < kLookWindow; ++j)
          w[j] = t - j >= 0 ? ldVolatile(lookback + (size_t)(t - j) * kRadix + b) : 0u;
        int used = 0;
#pragma unroll
        for (int j = 0; j < kLookWindow; ++j) {
          if (done || used < j) continue;  // stopped at an unpublished tile
          const unsigned flag = w[j] & ~kValueMask;
          if (flag == 0u) continue;
          excl += w[j] & kValueMask;
          used = j + 1;
          if (flag == kFlagPrefix) done = true;
        }
        if (done) break;
        t -= used;  // t >= 0: tile 0 publishes a prefix, so the walk stops there
        if (used == 0 && ++empty > 64) __nanosleep(64);
      }
      stVolatile(row + b, kFlagPrefix | ((excl + count) & kValueMask));
    }
  }

  unsigned digitStart = blockExclusiveScan<THREADS>(owner ? __ldg(hist + b) : 0u, sWarpSums);
  unsigned binExcl = blockExclusiveScan<THREADS>(count, sWarpSums);
  if (owner) {
    sBinExcl[b] = binExcl;
    sBase[b] = (int)(digitStart + excl) - (int)binExcl;
  }
  __syncthreads();

  // Stage the tile in digit order.
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    unsigned idx = wbase + r * 32 + lane;
    if (idx < n) {
      unsigned d = (key[r] >> shift) & (kRadix - 1);
      unsigned lp = sBinExcl[d] + sWarpHist[warp][d] + rank[r];
      sKeys[lp] = key[r];
      sVals[lp] = val[r];
    }
  }
  __syncthreads();

  // Write out: consecutive staged slots of one digit go to consecutive
  // global positions.
  unsigned tileCount = n - base < (unsigned)kTileKeys ? n - base : (unsigned)kTileKeys;
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    unsigned lp = r * THREADS + tid;
    if (lp < tileCount) {
      unsigned k = sKeys[lp];
      unsigned d = (k >> shift) & (kRadix - 1);
      unsigned g = (unsigned)(sBase[d] + (int)lp);
      if (g < n) {  // always true unless a look-back wait timed out
        keysOut[g] = k;
        valsOut[g] = sVals[lp];
      }
    }
  }
}

// The pass configurations the tuner chooses from.
struct PassConfig {
  int threads, items;
  size_t smem;
  void (*kernel)(const unsigned *, const unsigned *, unsigned *, unsigned *, unsigned, int,
                 const unsigned *, unsigned *, unsigned *, unsigned *, unsigned);
  int tile() const { return threads * items; }
};

template <int T, int I, int B>
constexpr PassConfig passConfig() {
  return PassConfig{T, I, onesweepSmem<T, I>(), &kOnesweep<T, I, B>};
}

const PassConfig kPassConfigs[] = {
    passConfig<256, 16, 2>(),  // 0: the fixed configuration
    passConfig<256, 12, 2>(),  // 1
    passConfig<256, 8, 3>(),   // 2
    passConfig<512, 8, 1>(),   // 3
    passConfig<512, 6, 2>(),   // 4
    passConfig<256, 20, 1>(),  // 5
};
constexpr int kNumPassConfigs = sizeof(kPassConfigs) / sizeof(kPassConfigs[0]);

// Tuned choice per size class (log2 of the particle count); -1 = default.
int g_sortChoice[33];
bool g_sortChoiceInit = false;
std::mutex g_sortChoiceMutex;

// Opts a configuration's kernel into its dynamic shared memory size (once per
// device).
bool prepareConfig(const PassConfig &pc) {
  static bool done[64][kNumPassConfigs] = {};
  int dev = 0;
  if (!cudaOk(cudaGetDevice(&dev))) return false;
  if (dev < 0 || dev >= 64) dev = 0;
  int idx = (int)(&pc - kPassConfigs);
  if (done[dev][idx]) return true;
  if (!cudaOk(cudaFuncSetAttribute(pc.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)pc.smem)))
    return false;
  done[dev][idx] = true;
  return true;
}

int sizeClass(unsigned n) {
  int c = 0;
  while ((1u << c) < n && c < 32) ++c;
  return c;
}

const PassConfig &chooseConfig(unsigned n) {
  std::lock_guard<std::mutex> lock(g_sortChoiceMutex);
  if (!g_sortChoiceInit) {
    for (int &v : g_sortChoice) v = -1;
    g_sortChoiceInit = true;
  }
  int k = g_sortChoice[sizeClass(n)];
  return kPassConfigs[k >= 0 && k < kNumPassConfigs ? k : 0];
}

inline size_t alignUp(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

void radixSortPairs(Context &c, unsigned *keys, unsigned *vals, unsigned n,
                    int bits, bool identityVals) {
  if (n < 2) return;
  if (n > kValueMask) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (bits < 1) bits = 1;
  if (bits > 32) bits = 32;
  const int passes = (bits + kRadixBits - 1) / kRadixBits;
  const PassConfig &pc = chooseConfig(n);
  if (!prepareConfig(pc)) return;
  const unsigned tiles = (n + pc.tile() - 1) / pc.tile();
  const size_t arr = alignUp((size_t)n * 4);
  const size_t histBytes = alignUp(kMaxPasses * kRadix * 4 + kMaxPasses * 4);
  const size_t lbBytes = alignUp((size_t)passes * tiles * kRadix * 4);
  const int buffers = (passes % 2 == 1) ? 2 : 1;  // extra key/value pairs
  const size_t total = (size_t)buffers * 2 * arr + histBytes + lbBytes;
  char *s = (char *)scratch(c, total);
  if (!s) return;
  unsigned *kB = (unsigned *)s, *vB = (unsigned *)(s + arr);
  unsigned *kC = buffers > 1 ? (unsigned *)(s + 2 * arr) : nullptr;
  unsigned *vC = buffers > 1 ? (unsigned *)(s + 3 * arr) : nullptr;
  char *meta = s + (size_t)buffers * 2 * arr;
  unsigned *hist = (unsigned *)meta;
  unsigned *counters = hist + kMaxPasses * kRadix;
  unsigned *lookback = (unsigned *)(meta + histBytes);
  cudaStream_t st = curStream();

  if (!cudaOk(cudaMemsetAsync(meta, 0, histBytes + lbBytes, st))) return;
  unsigned upBlocks = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (upBlocks > numSms() * 4u) upBlocks = numSms() * 4u;
  kUpsweep<<<upBlocks, kThreads, 0, st>>>(keys, n, passes, bits, hist, c.dStatus);
  if (!launchOk()) return;

  // Buffer routing: even pass counts alternate A->B->A; odd counts >= 3 go
  // A->B->C->A first so that the result lands in the caller's arrays.
  unsigned *srcK = keys, *srcV = identityVals ? nullptr : vals;
  for (int p = 0; p < passes; ++p) {
    unsigned *dstK, *dstV;
    if (passes == 1) {
      dstK = kB; dstV = vB;
    } else if (passes % 2 == 1 && p < 3) {
      if (p == 0) { dstK = kB; dstV = vB; }
      else if (p == 1) { dstK = kC; dstV = vC; }
      else { dstK = keys; dstV = vals; }
    } else {
      bool toB = (srcK == keys);
      dstK = toB ? kB : keys;
      dstV = toB ? vB : vals;
    }
    pc.kernel<<<tiles, pc.threads, pc.smem, st>>>(
        srcK, srcV, dstK, dstV, n, p * kRadixBits, hist + p * kRadix,
        lookback + (size_t)p * tiles * kRadix, counters + p, c.dStatus, sortWaitLimit());
    if (!launchOk()) return;
    srcK = dstK;
    srcV = dstV;
  }
  if (srcK != keys) {  // single pass: copy back
    cudaOk(cudaMemcpyAsync(keys, srcK, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
    cudaOk(cudaMemcpyAsync(vals, srcV, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  }
}


// ---------------------------------------------------------------------------
// sortParticles without allocation (fcdemSortParticlesNoAlloc).
//
// Some callers must not have the library allocate device memory: hosts that
// own every byte of device memory through their own pool and forbid hidden
// allocations, and loops running close to the memory limit, where a
// cudaMalloc in the middle of a step can fail.  sortParticles grows its
// scratch with cudaMalloc on first use; this variant uses a fixed scratch
// array in the library's static device memory instead, sized for
// kNoAllocMaxParticles particles.  That array exists on every GPU that loads
// the library, for the life of the process.

namespace {

constexpr unsigned kNoAllocMaxParticles = 1u << 20;
constexpr size_t kNoAllocArr = (size_t)kNoAllocMaxParticles * 4;  // one key/value array
constexpr unsigned kNoAllocMaxTiles = (kNoAllocMaxParticles + kTile - 1) / kTile;
constexpr size_t kNoAllocHist = (kMaxPasses * kRadix * 4 + kMaxPasses * 4 + 255) & ~(size_t)255;
constexpr size_t kNoAllocLookback = (size_t)kMaxPasses * kNoAllocMaxTiles * kRadix * 4;
constexpr size_t kNoAllocStatus = 256;
constexpr size_t kNoAllocBytes =
    4 * kNoAllocArr + kNoAllocHist + kNoAllocLookback + kNoAllocStatus;  // ~17 MB

// The scratch itself.  In host code this name is only a host-side stand-in
// for the device array, not a device address: the kernels get the address
// that cudaGetSymbolAddress returns for the current device.  Its last 256
// bytes hold the sort's own status word (kStatus* bits), read and cleared
// by fcdemGetLastError like the context's.
static __device__ __align__(256) unsigned char g_noAllocScratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noAllocMutex;
unsigned char *g_noAllocPtr[kNoAllocMaxDevices] = {};

unsigned *statusIn(unsigned char *scratch) {
  return (unsigned *)(scratch + 4 * kNoAllocArr + kNoAllocHist + kNoAllocLookback);
}

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached, its status word cleared
// then; nullptr on failure.
unsigned char *noAllocScratch() {
  int dev = 0;
  if (!cudaOk(cudaGetDevice(&dev))) return nullptr;
  if (dev < 0 || dev >= kNoAllocMaxDevices) { setError(FCDEM_ERR_INVALID_VALUE); return nullptr; }
  std::lock_guard<std::mutex> lock(g_noAllocMutex);
  if (!g_noAllocPtr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noAllocScratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      setError(FCDEM_ERR_CUDA);
      return nullptr;
    }
    if (!cudaOk(cudaMemset(statusIn((unsigned char *)p), 0, sizeof(unsigned)))) return nullptr;
    g_noAllocPtr[dev] = (unsigned char *)p;
  }
  return g_noAllocPtr[dev];
}

}  // namespace

unsigned *noAllocStatusWord() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_noAllocMutex);
  return g_noAllocPtr[dev] ? statusIn(g_noAllocPtr[dev]) : nullptr;
}

unsigned sortWaitLimit() { return g_sortWaitRounds.load(std::memory_order_relaxed); }

}  // namespace fcdem

extern "C" void fcdemSetSortWaitLimit(int rounds) {
  fcdem::g_sortWaitRounds.store(rounds < 0 ? fcdem::kSortWaitRounds : (unsigned)rounds);
}

extern "C" void fcdemSortParticlesNoAlloc(uint *dGridParticleHash, uint *dGridParticleIndex,
                                          uint numParticles) {
  using namespace fcdem;
  const unsigned n = numParticles;
  if (n < 2) return;
  if (!dGridParticleHash || !dGridParticleIndex) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (n > kNoAllocMaxParticles) {  // the fixed scratch does not fit more
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  unsigned char *s = noAllocScratch();
  if (!s) return;
  if (!prepareConfig(kPassConfigs[0])) return;  // 40 KB dynamic shared memory: fits the default
  // Same key width as sortParticles when setParameters has been called on
  // this device (all 32 bits otherwise); no context is created here.
  SimParams params;
  const int bits = paramsIfSet(params) ? keyBits(params.numCells) : 32;
  const int passes = (bits + kRadixBits - 1) / kRadixBits;
  const unsigned tiles = (n + kTile - 1) / kTile;
  unsigned *keys = dGridParticleHash, *vals = dGridParticleIndex;
  unsigned *kB = (unsigned *)s, *vB = (unsigned *)(s + kNoAllocArr);
  unsigned *kC = (unsigned *)(s + 2 * kNoAllocArr), *vC = (unsigned *)(s + 3 * kNoAllocArr);
  unsigned char *meta = s + 4 * kNoAllocArr;
  unsigned *hist = (unsigned *)meta;
  unsigned *counters = hist + kMaxPasses * kRadix;
  unsigned *lookback = (unsigned *)(meta + kNoAllocHist);
  unsigned *status = statusIn(s);
  cudaStream_t st = curStream();
  // The array keeps whatever the previous call left; the histograms, tile
  // counters and look-back flags must start at zero.  (The status word is
  // not cleared here: it holds the bits of earlier calls until
  // fcdemGetLastError reads them.)
  if (!cudaOk(cudaMemsetAsync(meta, 0, kNoAllocHist + (size_t)passes * tiles * kRadix * 4,
                              st)))
    return;
  unsigned upBlocks = (n + kThreads * 16 - 1) / (kThreads * 16);
  if (upBlocks > numSms() * 4u) upBlocks = numSms() * 4u;
  kUpsweep<<<upBlocks, kThreads, 0, st>>>(keys, n, passes, bits, hist, status);
  if (!launchOk()) return;
  unsigned *srcK = keys, *srcV = vals;
  for (int p = 0; p < passes; ++p) {
    unsigned *dstK, *dstV;
    if (passes == 1) {
      dstK = kB; dstV = vB;
    } else if (passes % 2 == 1 && p < 3) {
      if (p == 0) { dstK = kB; dstV = vB; }
      else if (p == 1) { dstK = kC; dstV = vC; }
      else { dstK = keys; dstV = vals; }
    } else {
      bool toB = (srcK == keys);
      dstK = toB ? kB : keys;
      dstV = toB ? vB : vals;
    }
    kOnesweep<kThreads, kItems, 2><<<tiles, kThreads, onesweepSmem<kThreads, kItems>(), st>>>(
        srcK, srcV, dstK, dstV, n, p * kRadixBits, hist + p * kRadix,
        lookback + (size_t)p * tiles * kRadix, counters + p, status, sortWaitLimit());
    if (!launchOk()) return;
    srcK = dstK;
    srcV = dstV;
  }
  if (srcK != keys) {
    cudaOk(cudaMemcpyAsync(keys, srcK, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
    cudaOk(cudaMemcpyAsync(vals, srcV, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  }
}

// ---------------------------------------------------------------------------
// Sort autotuner: times every pass configuration on uniformly distributed
// keys below numCells and keeps the fastest for this size class.

namespace fcdem {
namespace {
__global__ void kTuneKeys(unsigned *keys, unsigned *vals, unsigned n, unsigned mask,
                          unsigned numCells, unsigned salt) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned h = (i + salt) * 2654435761u;
  h ^= h >> 15;
  h *= 2246822519u;
  h ^= h >> 13;
  h &= mask;
  keys[i] = h < numCells ? h : h - numCells;
  vals[i] = i;
}
}  // namespace
}  // namespace fcdem

extern "C" int fcdemSetSortConfig(unsigned numParticles, int config) {
  using namespace fcdem;
  if (config < -1 || config >= kNumPassConfigs) { setError(FCDEM_ERR_INVALID_VALUE); return -1; }
  chooseConfig(numParticles);  // initialises the table
  std::lock_guard<std::mutex> lock(g_sortChoiceMutex);
  g_sortChoice[sizeClass(numParticles)] = config;
  return kNumPassConfigs;
}

extern "C" int fcdemAutotuneSort(unsigned numParticles, unsigned numCells, float *bestMs) {
  using namespace fcdem;
  const unsigned n = numParticles;
  if (n < 2 || numCells == 0) { setError(FCDEM_ERR_INVALID_VALUE); return -1; }
  Context &c = ctx();
  cudaStream_t st = curStream();
  unsigned *k0 = nullptr, *v0 = nullptr, *k1 = nullptr, *v1 = nullptr;
  if (cudaMalloc(&k0, (size_t)n * 16) != cudaSuccess) {
    cudaGetLastError();
    setError(FCDEM_ERR_ALLOC);
    return -1;
  }
  v0 = k0 + n;
  k1 = v0 + n;
  v1 = k1 + n;
  int bits = keyBits(numCells);
  unsigned mask = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
  kTuneKeys<<<(n + 255) / 256, 256, 0, st>>>(k0, v0, n, mask, numCells, 12345u);
  launchOk();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = 0;
  float bestT = 3.4e38f;
  for (int k = 0; k < kNumPassConfigs; ++k) {
    fcdemSetSortConfig(n, k);
    float tot = 0.0f;
    for (int rep = 0; rep < 4; ++rep) {
      cudaMemcpyAsync(k1, k0, (size_t)n * 8, cudaMemcpyDeviceToDevice, st);
      cudaEventRecord(e0, st);
      radixSortPairs(c, k1, v1, n, bits);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float t = 0.0f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) tot += t;  // the first run warms up
    }
    if (tot < bestT) { bestT = tot; best = k; }
  }
  fcdemSetSortConfig(n, best);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(k0);
  if (bestMs) *bestMs = bestT / 3.0f;
  return best;
}
