// fcdem_context.cu -- per-device state, error reporting and the support
// entry points of the reference's C interface (particleSystem.cu:36-127).
#include <atomic>
#include <cstdio>
#include <vector>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "fcdem_internal.cuh"

namespace fcdem {

namespace {
constexpr int kMaxDevices = 64;
Context g_ctx[kMaxDevices];
std::mutex g_mutex;
std::atomic<int> g_error{FCDEM_SUCCESS};
std::atomic<unsigned long long> g_launches{0};
thread_local cudaStream_t t_stream = nullptr;

struct Profiler {
  bool on = false;
  struct Pair { int stage; cudaEvent_t a, b; };
  std::vector<Pair> open;         // recorded, not yet read
  std::vector<cudaEvent_t> pool;  // free events
  int pending[FCDEM_NUM_STAGES] = {};
  cudaEvent_t begin[FCDEM_NUM_STAGES] = {};
  double totalMs[FCDEM_NUM_STAGES] = {};
  unsigned count[FCDEM_NUM_STAGES] = {};
  cudaEvent_t take() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaOk(cudaEventCreate(&e));
    return e;
  }
};
Profiler g_prof;
std::mutex g_prof_mutex;
}  // namespace

void stageBegin(int stage) {
  if (!g_prof.on || stage < 0 || stage >= FCDEM_NUM_STAGES) return;
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  cudaEvent_t e = g_prof.take();
  if (e && cudaOk(cudaEventRecord(e, t_stream))) g_prof.begin[stage] = e;
}

void stageEnd(int stage) {
  if (!g_prof.on || stage < 0 || stage >= FCDEM_NUM_STAGES) return;
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  cudaEvent_t a = g_prof.begin[stage];
  if (!a) return;
  g_prof.begin[stage] = nullptr;
  cudaEvent_t b = g_prof.take();
  if (b && cudaOk(cudaEventRecord(b, t_stream))) g_prof.open.push_back({stage, a, b});
}

cudaStream_t curStream() { return t_stream; }

void setError(int code) {
  int expected = FCDEM_SUCCESS;
  g_error.compare_exchange_strong(expected, code);
}

bool cudaOk(cudaError_t e) {
  if (e == cudaSuccess) return true;
  cudaGetLastError();  // clear a non-sticky error
  setError(FCDEM_ERR_CUDA);
  return false;
}

bool launchOk() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaOk(cudaGetLastError());
}

Context &ctx() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  if (dev < 0 || dev >= kMaxDevices) dev = 0;
  Context &c = g_ctx[dev];
  if (c.device < 0) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (c.device < 0) {
      unsigned *status = nullptr;
      if (cudaOk(cudaMalloc(&status, sizeof(unsigned))) &&
          cudaOk(cudaMemset(status, 0, sizeof(unsigned)))) {
        c.dStatus = status;
      }
      c.device = dev;
    }
  }
  return c;
}

bool paramsIfSet(SimParams &out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (dev < 0 || dev >= kMaxDevices) return false;
  std::lock_guard<std::mutex> lock(g_mutex);
  const Context &c = g_ctx[dev];
  if (c.device < 0 || !c.haveParams) return false;
  out = c.params;
  return true;
}

unsigned numSms() {
  static std::atomic<int> sms[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = -1;
  }
  if (dev >= 0 && dev < kMaxDevices) {
    int v = sms[dev].load(std::memory_order_relaxed);
    if (v > 0) return (unsigned)v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
        v > 0) {
      sms[dev].store(v, std::memory_order_relaxed);
      return (unsigned)v;
    }
    cudaGetLastError();
  }
  return 152u;  // GB300 (not reached on a working device)
}

void *scratch(Context &c, size_t bytes) {
  if (bytes <= c.scratchBytes) return c.scratch;
  // Work already queued (on any stream) may still use the old block.
  if (!cudaOk(cudaDeviceSynchronize())) return nullptr;
  if (c.scratch) cudaFree(c.scratch);
  c.scratch = nullptr;
  c.scratchBytes = 0;
  size_t grown = bytes + bytes / 4;
  if (cudaMalloc(&c.scratch, grown) != cudaSuccess) {
    cudaGetLastError();
    c.scratch = nullptr;
    setError(FCDEM_ERR_ALLOC);
    return nullptr;
  }
  c.scratchBytes = grown;
  return c.scratch;
}

bool mortonUsable(const SimParams &p) {
  return p.gridSize[0] == p.gridSize[1] && p.gridSize[1] == p.gridSize[2] &&
         p.gridSize[0] >= 1u && p.gridSize[0] <= 1024u;
}

KParams kparams(const Context &c) {
  KParams k;
  k.p = c.params;
  k.p.maxParticlesPerCell = (c.morton && mortonUsable(c.params)) ? kMortonTag : 0u;
  k.radiusFromW = c.radiusFromW;
  return k;
}

}  // namespace fcdem

using namespace fcdem;

extern "C" {

void cudaInit(int argc, char **argv) {
  int dev = 0;
  for (int i = 1; i < argc && argv; ++i) {
    const char *a = argv[i];
    if (!a) continue;
    while (*a == '-') ++a;
    if (std::strncmp(a, "device=", 7) == 0) dev = std::atoi(a + 7);
  }
  int count = 0;
  if (!cudaOk(cudaGetDeviceCount(&count)) || count == 0) {
    setError(FCDEM_ERR_CUDA);
    return;
  }
  if (dev < 0 || dev >= count) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  cudaOk(cudaSetDevice(dev));
}

void allocateArray(void **devPtr, int size) {
  if (!devPtr || size < 0) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (cudaMalloc(devPtr, (size_t)size) != cudaSuccess) {
    cudaGetLastError();
    *devPtr = nullptr;
    setError(FCDEM_ERR_ALLOC);
  }
}

void freeArray(void *devPtr) { cudaOk(cudaFree(devPtr)); }

void threadSync(void) { cudaOk(cudaDeviceSynchronize()); }

void copyArrayFromDevice(void *host, const void *device,
                         struct cudaGraphicsResource **cuda_vbo_resource,
                         int size) {
  if (cuda_vbo_resource && *cuda_vbo_resource) {
    setError(FCDEM_ERR_UNSUPPORTED);
    return;
  }
  if (size < 0) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  cudaStream_t s = curStream();
  if (cudaOk(cudaMemcpyAsync(host, device, (size_t)size, cudaMemcpyDeviceToHost, s)))
    cudaOk(cudaStreamSynchronize(s));
}

void copyArrayToDevice(void *device, const void *host, int offset, int size) {
  if (size < 0 || offset < 0) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  cudaStream_t s = curStream();
  if (cudaOk(cudaMemcpyAsync((char *)device + offset, host, (size_t)size,
                             cudaMemcpyHostToDevice, s)))
    cudaOk(cudaStreamSynchronize(s));
}

void registerGLBufferObject(uint, struct cudaGraphicsResource **) {
  setError(FCDEM_ERR_UNSUPPORTED);
}
void unregisterGLBufferObject(struct cudaGraphicsResource *) {
  setError(FCDEM_ERR_UNSUPPORTED);
}
void *mapGLBufferObject(struct cudaGraphicsResource **) {
  setError(FCDEM_ERR_UNSUPPORTED);
  return nullptr;
}
void unmapGLBufferObject(struct cudaGraphicsResource *) {
  setError(FCDEM_ERR_UNSUPPORTED);
}

void setParameters(SimParams *hostParams) {
  if (!hostParams) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  Context &c = ctx();
  std::lock_guard<std::mutex> lock(g_mutex);
  c.params = *hostParams;
  c.haveParams = true;
}

}  // extern "C"

namespace {
// Reads and clears a device status word (synchronising the library stream)
// and records the first error its bits stand for.
void drainStatus(unsigned *word) {
  unsigned status = 0;
  cudaStream_t s = curStream();
  if (cudaMemcpyAsync(&status, word, sizeof(unsigned), cudaMemcpyDeviceToHost, s) ==
          cudaSuccess &&
      cudaStreamSynchronize(s) == cudaSuccess) {
    if (status) {
      cudaMemsetAsync(word, 0, sizeof(unsigned), s);
      if (status & kStatusTimeout) setError(FCDEM_ERR_DEVICE_TIMEOUT);
      else if (status & kStatusKeyRange) setError(FCDEM_ERR_KEY_RANGE);
      else if (status & kStatusRadiusBound) setError(FCDEM_ERR_RADIUS_BOUND);
      else if (status & kStatusCellOverflow) setError(FCDEM_ERR_CELL_OVERFLOW);
    }
  } else {
    cudaGetLastError();
    setError(FCDEM_ERR_CUDA);
  }
}
}  // namespace

extern "C" {

int fcdemGetLastError(void) {
  Context &c = ctx();
  if (c.dStatus) drainStatus(c.dStatus);
  // the allocation-free sort keeps its own status word in its static scratch
  if (unsigned *w = noAllocStatusWord()) drainStatus(w);
  return g_error.exchange(FCDEM_SUCCESS);
}

const char *fcdemGetErrorString(int code) {
  switch (code) {
    case FCDEM_SUCCESS: return "no error";
    case FCDEM_ERR_INVALID_VALUE: return "invalid argument";
    case FCDEM_ERR_CUDA: return "a CUDA runtime call failed";
    case FCDEM_ERR_NO_PARAMS: return "setParameters has not been called";
    case FCDEM_ERR_UNSUPPORTED: return "OpenGL interop is not supported";
    case FCDEM_ERR_DEVICE_TIMEOUT: return "a bounded device-side wait expired";
    case FCDEM_ERR_KEY_RANGE: return "sort key above the grid's key width";
    case FCDEM_ERR_ALLOC: return "device allocation failed";
    case FCDEM_ERR_CELL_OVERFLOW:
      return "fcdemUpdate: the list of crowded cells overflowed (order inside a cell not stable)";
    case FCDEM_ERR_RADIUS_BOUND:
      return "radius-from-w mode: a particle radius exceeds SimParams.particleRadius";
    default: return "unknown error";
  }
}

void fcdemSetStream(void *stream) { t_stream = (cudaStream_t)stream; }

void fcdemSetRadiusMode(int radiusFromW) { ctx().radiusFromW = radiusFromW ? 1 : 0; }

void fcdemSetCellOrder(int morton) { ctx().morton = morton ? 1 : 0; }

const char *fcdemVersion(void) { return "fcdem-gb300 0.1 (sm_103a)"; }

unsigned long long fcdemGetLaunchCount(void) { return g_launches.load(); }

void fcdemSetProfiling(int on) {
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  for (auto &p : g_prof.open) { g_prof.pool.push_back(p.a); g_prof.pool.push_back(p.b); }
  g_prof.open.clear();
  for (int k = 0; k < FCDEM_NUM_STAGES; ++k) {
    if (g_prof.begin[k]) g_prof.pool.push_back(g_prof.begin[k]);
    g_prof.begin[k] = nullptr;
    g_prof.totalMs[k] = 0.0;
    g_prof.count[k] = 0;
  }
  g_prof.on = on != 0;
}

int fcdemGetStageTimes(float *ms, unsigned *launches, int maxStages) {
  std::lock_guard<std::mutex> lock(g_prof_mutex);
  for (auto &p : g_prof.open) {
    float t = 0.0f;
    if (cudaOk(cudaEventSynchronize(p.b)) && cudaOk(cudaEventElapsedTime(&t, p.a, p.b))) {
      g_prof.totalMs[p.stage] += t;
      g_prof.count[p.stage] += 1;
    }
    g_prof.pool.push_back(p.a);
    g_prof.pool.push_back(p.b);
  }
  g_prof.open.clear();
  for (int k = 0; k < FCDEM_NUM_STAGES && k < maxStages; ++k) {
    if (ms) ms[k] = (float)g_prof.totalMs[k];
    if (launches) launches[k] = g_prof.count[k];
  }
  return FCDEM_NUM_STAGES;
}

}  // extern "C"
