/*
 * refgpu_loader.cpp -- TEST INFRASTRUCTURE.  Loads
 * oracle/_ref/fcref_kernels.cubin (the reference's own kernels, see
 * refgpu.cu) with the CUDA driver API and launches them with the launch glue
 * of cuda_addon/particleSystem.cu:135-270 restated: 256 threads per block for
 * calcHash and reorder, 64 for collide, a 0xff memset of cellStart before
 * the reorder, (blockDim + 1) * 4 bytes of dynamic shared memory for it, and
 * the parameter block copied into the module's __constant__ `params`
 * (particleSystem.cu:123-127).  All pointers are device pointers; launches go
 * to the given stream (0 = legacy default stream).
 */
#include <cuda.h>

#include <algorithm>
#include <cstddef>

namespace {
CUmodule g_mod = nullptr;
CUfunction g_integrate = nullptr, g_hash = nullptr, g_reorder = nullptr,
           g_collide = nullptr;
CUdeviceptr g_params = 0;
size_t g_params_bytes = 0;

int ensure_context() {
  if (cuInit(0) != CUDA_SUCCESS) return 1;
  CUcontext ctx = nullptr;
  if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS) return 2;
  if (ctx) return 0;
  CUdevice dev;
  if (cuDeviceGet(&dev, 0) != CUDA_SUCCESS) return 3;
  if (cuDevicePrimaryCtxRetain(&ctx, dev) != CUDA_SUCCESS) return 4;
  return cuCtxSetCurrent(ctx) == CUDA_SUCCESS ? 0 : 5;
}

void grid_size(unsigned n, unsigned block, unsigned &nb, unsigned &nt) {
  nt = std::min(block, n);
  nb = nt ? (n + nt - 1) / nt : 0;
}

int launch(CUfunction f, unsigned nb, unsigned nt, unsigned smem, void *stream,
           void **args) {
  if (nb == 0) return 0;
  CUresult r = cuLaunchKernel(f, nb, 1, 1, nt, 1, 1, smem, (CUstream)stream,
                              args, nullptr);
  return r == CUDA_SUCCESS ? 0 : 100 + (int)r;
}
}  // namespace

extern "C" {

/* Returns 0 on success. */
int fcrefgpu_load(const char *cubin_path) {
  if (g_mod) return 0;
  int e = ensure_context();
  if (e) return e;
  if (cuModuleLoad(&g_mod, cubin_path) != CUDA_SUCCESS) return 10;
  /* Itanium-mangled names of the reference's __global__ functions. */
  if (cuModuleGetFunction(&g_hash, g_mod, "_Z9calcHashDPjS_P6float4j") != CUDA_SUCCESS)
    return 11;
  if (cuModuleGetFunction(&g_reorder, g_mod,
                          "_Z28reorderDataAndFindCellStartDPjS_P6float4S1_S_S_S1_S1_j") !=
      CUDA_SUCCESS)
    return 12;
  if (cuModuleGetFunction(&g_collide, g_mod, "_Z8collideDP6float4S0_S0_PjS1_S1_j") !=
      CUDA_SUCCESS)
    return 13;
  if (cuModuleGetFunction(&g_integrate, g_mod, "fcref_integrate") != CUDA_SUCCESS)
    return 14;
  if (cuModuleGetGlobal(&g_params, &g_params_bytes, g_mod, "params") != CUDA_SUCCESS)
    return 15;
  return 0;
}

int fcrefgpu_params_bytes(void) { return (int)g_params_bytes; }

int fcrefgpu_set_parameters(const void *host_params) {
  if (!g_mod) return 20;
  return cuMemcpyHtoD(g_params, host_params, g_params_bytes) == CUDA_SUCCESS ? 0 : 21;
}

int fcrefgpu_integrate(CUdeviceptr pos, CUdeviceptr vel, float dt, unsigned n,
                       void *stream) {
  unsigned nb, nt;
  grid_size(n, 256, nb, nt);
  void *args[] = {&pos, &vel, &dt, &n};
  return launch(g_integrate, nb, nt, 0, stream, args);
}

int fcrefgpu_calc_hash(CUdeviceptr hash, CUdeviceptr index, CUdeviceptr pos,
                       unsigned n, void *stream) {
  unsigned nb, nt;
  grid_size(n, 256, nb, nt);
  void *args[] = {&hash, &index, &pos, &n};
  return launch(g_hash, nb, nt, 0, stream, args);
}

int fcrefgpu_reorder(CUdeviceptr cellStart, CUdeviceptr cellEnd,
                     CUdeviceptr sortedPos, CUdeviceptr sortedVel,
                     CUdeviceptr hash, CUdeviceptr index, CUdeviceptr oldPos,
                     CUdeviceptr oldVel, unsigned n, unsigned numCells,
                     void *stream) {
  if (cuMemsetD8Async(cellStart, 0xff, (size_t)numCells * 4, (CUstream)stream) !=
      CUDA_SUCCESS)
    return 30;
  unsigned nb, nt;
  grid_size(n, 256, nb, nt);
  void *args[] = {&cellStart, &cellEnd, &sortedPos, &sortedVel, &hash,
                  &index,     &oldPos,  &oldVel,    &n};
  return launch(g_reorder, nb, nt, (nt + 1) * 4, stream, args);
}

int fcrefgpu_collide(CUdeviceptr newVel, CUdeviceptr sortedPos,
                     CUdeviceptr sortedVel, CUdeviceptr index,
                     CUdeviceptr cellStart, CUdeviceptr cellEnd, unsigned n,
                     void *stream) {
  unsigned nb, nt;
  grid_size(n, 64, nb, nt);
  void *args[] = {&newVel, &sortedPos, &sortedVel, &index,
                  &cellStart, &cellEnd, &n};
  return launch(g_collide, nb, nt, 0, stream, args);
}

int fcrefgpu_sync(void) {
  return cuCtxSynchronize() == CUDA_SUCCESS ? 0 : 40;
}

}  // extern "C"
