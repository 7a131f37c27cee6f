// fcdem_sdf.cu -- neural signed-distance field of an obstacle, used to cull
// the distance-map boundary test (boundaries.cuh:38-63) for particles far
// from the obstacle.  No counterpart in the reference: the map query stays
// the fallback inside the skin band and the judge of the network's error.
//
// Network: inputs (x, y, z) normalised to the obstacle box, optionally with a
// one-hot shape code; `layers` hidden SiLU layers of width `hidden`; one
// linear output, the distance divided by outScale.  Parameters, FP32, in one
// vector: W0 [H][D], b0 [H], then per further hidden layer W [H][H], b [H],
// then wOut [H], bOut.  Weight matrices are row-major [out][in].
//
//  * training (FP32): kSdfTrain runs forward and backward for a tile of S
//    samples per CTA with every activation in shared memory; the products are
//    4x4 register tiles over shared-memory operands; the tile's weight and
//    bias gradients are added to the batch gradient with atomics; kSdfAdam
//    applies Adam and refreshes the transposed weight copies the forward
//    reads;
//  * inference (BF16 weights and activations, FP32 accumulate): kSdfInfer
//    and the culled integrate give each CTA 128 points.  The first layer
//    (3 or 11 inputs) and the output layer run on the CUDA cores; each H x H
//    hidden layer is one tcgen05.mma chain (M = 128 points, N = H, K = H in
//    steps of 16) from shared-memory operands into a TMEM accumulator, read
//    back with tcgen05.ld for the bias + SiLU epilogue, which writes the next
//    layer's operand tile.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "fcdem_map.cuh"

namespace fcdem {
namespace {

constexpr int kSdfMaxInputs = 16;  // 3 coordinates + up to 13 shape codes
constexpr unsigned kSdfWaitLimit = 1u << 22;

struct SdfLayout {
  int D, H, L;              // inputs, width, hidden layers (1..3)
  unsigned w0, b0;          // first layer
  unsigned wh[2], bh[2];    // further hidden layers 1 .. L-1
  unsigned wo, bo;          // output layer
  unsigned total;
};

SdfLayout makeLayout(int D, int H, int L) {
  SdfLayout s{};
  s.D = D;
  s.H = H;
  s.L = L;
  unsigned o = 0;
  s.w0 = o;
  o += (unsigned)(H * D);
  s.b0 = o;
  o += (unsigned)H;
  for (int l = 1; l < L; ++l) {
    s.wh[l - 1] = o;
    o += (unsigned)(H * H);
    s.bh[l - 1] = o;
    o += (unsigned)H;
  }
  s.wo = o;
  o += (unsigned)H;
  s.bo = o;
  o += 1;
  s.total = o;
  return s;
}

// What the kernels read of a network.
struct SdfView {
  SdfLayout lay;
  const float *__restrict__ p;   // parameters
  const float *__restrict__ pT;  // same, weight matrices transposed ([in][out])
  const __nv_bfloat16 *__restrict__ w16;  // hidden layers 1..L-1, tensor-core tiles
  float shift[3], scale[3], outScale;
};

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
// Inference SiLU: silu(z) = h + h tanh(h) with h = z / 2, the hardware
// tanh approximation (one special-function op; relative error about 2^-11,
// near the bf16 rounding of the activations it feeds).  The culling
// threshold is calibrated on this arithmetic (the prediction the kernels
// make), so its error is part of what the exact map judges.
__device__ __forceinline__ float tanhApprox(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float siluFast(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanhApprox(h), h);
}
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.0f + z * (1.0f - s));
}

// splitmix64 stream: value number k of stream `seed`
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float uniform01(unsigned long long seed, unsigned long long k) {
  return (float)(mix64(seed + 0x9e3779b97f4a7c15ull * (k + 1)) >> 40) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------------------
// Training samples: (x, y, z, d) with d the map's trilinear distance
// (queryMap, the value the boundary test uses).  Sample t < nNear is drawn
// until |d| < band (at most 64 draws; the last draw is kept otherwise), the
// others uniformly in the map box.
__global__ void __launch_bounds__(256)
kSdfSamples(MapView M, float4 *__restrict__ out, int *__restrict__ shapeOut, int shape,
            unsigned n, unsigned nNear, float band, unsigned long long seed) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int tries = t < nNear ? 64 : 1;
  float3 q = make_float3(0.0f, 0.0f, 0.0f);
  float d = 0.0f;
  for (int a = 0; a < tries; ++a) {
    const unsigned long long k = ((unsigned long long)t * 64u + (unsigned)a) * 3u;
    q = make_float3(M.vmin.x + (M.vmax.x - M.vmin.x) * uniform01(seed, k),
                    M.vmin.y + (M.vmax.y - M.vmin.y) * uniform01(seed, k + 1),
                    M.vmin.z + (M.vmax.z - M.vmin.z) * uniform01(seed, k + 2));
    float3 cp;
    d = queryMap(M, q, cp);
    if (fabsf(d) < band) break;
  }
  out[t] = make_float4(q.x, q.y, q.z, d);
  if (shapeOut) shapeOut[t] = shape;
}

// ---------------------------------------------------------------------------
// Training: forward (+ backward) of S = 4096 / H samples per CTA.

// out[s][j] = bias[j] + sum_k in[s][k] * Wt[k][j] for the S x H tile; thread
// t owns rows 4*(t / (H/4)) .. +3 and columns 4*(t % (H/4)) .. +3.
template <int H>
__device__ __forceinline__ void gemmTile(const float *in, int inStride, int K,
                                         const float *__restrict__ Wt,
                                         const float *__restrict__ bias, float *out) {
  const int t = threadIdx.x;
  const int j0 = (t % (H / 4)) * 4, s0 = (t / (H / 4)) * 4;
  float acc[4][4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const float b = bias ? __ldg(bias + j0 + v) : 0.0f;
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u][v] = b;
  }
  for (int k = 0; k < K; ++k) {
    const float4 w = __ldg(reinterpret_cast<const float4 *>(Wt + (size_t)k * H + j0));
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float a = in[(s0 + u) * inStride + k];
      acc[u][0] = fmaf(a, w.x, acc[u][0]);
      acc[u][1] = fmaf(a, w.y, acc[u][1]);
      acc[u][2] = fmaf(a, w.z, acc[u][2]);
      acc[u][3] = fmaf(a, w.w, acc[u][3]);
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) out[(s0 + u) * H + j0 + v] = acc[u][v];
}

// g[j][k] += sum_s delta[s][j] * act[s][k] over the tile (k < K, act row
// stride actStride), then bias g_b[j] += sum_s delta[s][j].
template <int H>
__device__ __forceinline__ void weightGrad(const float *delta, const float *act, int actStride,
                                           int K, int S, float *__restrict__ gW,
                                           float *__restrict__ gB) {
  const int t = threadIdx.x;
  if ((K & 3) == 0) {
    const int tiles = (H / 4) * (K / 4);
    for (int e = t; e < tiles; e += blockDim.x) {
      const int j0 = (e / (K / 4)) * 4, k0 = (e % (K / 4)) * 4;
      float acc[4][4] = {};
      for (int s = 0; s < S; ++s) {
        float dj[4], ak[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          dj[u] = delta[s * H + j0 + u];
          ak[u] = act[s * actStride + k0 + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(dj[u], ak[v], acc[u][v]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) atomicAdd(gW + (j0 + u) * K + k0 + v, acc[u][v]);
    }
  } else {
    for (int e = t; e < H * K; e += blockDim.x) {
      const int j = e / K, k = e % K;
      float acc = 0.0f;
      for (int s = 0; s < S; ++s) acc = fmaf(delta[s * H + j], act[s * actStride + k], acc);
      atomicAdd(gW + e, acc);
    }
  }
  for (int j = t; j < H; j += blockDim.x) {
    float acc = 0.0f;
    for (int s = 0; s < S; ++s) acc += delta[s * H + j];
    atomicAdd(gB + j, acc);
  }
}

template <int H, int L>
constexpr size_t trainSmemBytes() {
  constexpr int S = 4096 / H;
  return sizeof(float) * ((size_t)S * kSdfMaxInputs + 2 * (size_t)L * S * H + 2 * (size_t)S * H +
                          2 * (size_t)S);
}

// Sample s of the tile is samples[base + s]: input (x - shift) * scale and
// the one-hot shape code, target d / outScale, weight 1 + 9 [|d| < band].
// kBackward: adds invB * the gradient of sum_s w (y - t)^2 to grad and the
// loss term to *loss; otherwise writes the distance prediction to yOut.
template <int H, int L, bool kBackward>
__global__ void __launch_bounds__(256)
kSdfTrain(SdfView net, const float4 *__restrict__ samples, const int *__restrict__ shapes,
          unsigned n, float band, float invB, float *__restrict__ grad, float *__restrict__ loss,
          float *__restrict__ yOut) {
  constexpr int S = 4096 / H;
  extern __shared__ __align__(16) float smf[];
  float *X = smf;                              // [S][kSdfMaxInputs]
  float *Z = X + S * kSdfMaxInputs;            // [L][S][H] pre-activations
  float *A = Z + L * S * H;                    // [L][S][H] activations
  float *D0 = A + L * S * H;                   // [S][H] deltas
  float *D1 = D0 + S * H;
  float *yv = D1 + S * H;                      // [S]
  float *dyv = yv + S;                         // [S]
  const SdfLayout &ly = net.lay;
  const int D = ly.D;
  const int t = threadIdx.x;
  const unsigned base = blockIdx.x * S;
  for (int e = t; e < S * kSdfMaxInputs; e += blockDim.x) {
    const int s = e / kSdfMaxInputs, d = e % kSdfMaxInputs;
    const unsigned idx = base + s;
    float v = 0.0f;
    if (idx < n && d < D) {
      const float4 q = __ldg(samples + idx);
      if (d < 3)
        v = ((d == 0 ? q.x : (d == 1 ? q.y : q.z)) - net.shift[d]) * net.scale[d];
      else
        v = (shapes && __ldg(shapes + idx) == d - 3) ? 1.0f : 0.0f;
    }
    X[e] = v;
  }
  __syncthreads();
  gemmTile<H>(X, kSdfMaxInputs, D, net.pT + ly.w0, net.p + ly.b0, Z);
  __syncthreads();
  for (int e = t; e < S * H; e += blockDim.x) A[e] = silu(Z[e]);
  __syncthreads();
  for (int l = 1; l < L; ++l) {
    gemmTile<H>(A + (l - 1) * S * H, H, H, net.pT + ly.wh[l - 1], net.p + ly.bh[l - 1],
                Z + l * S * H);
    __syncthreads();
    for (int e = t; e < S * H; e += blockDim.x) A[l * S * H + e] = silu(Z[l * S * H + e]);
    __syncthreads();
  }
  const float *AL = A + (L - 1) * S * H;
  for (int s = t; s < S; s += blockDim.x) {
    float y = __ldg(net.p + ly.bo);
    for (int k = 0; k < H; ++k) y = fmaf(AL[s * H + k], __ldg(net.p + ly.wo + k), y);
    yv[s] = y;
    const unsigned idx = base + s;
    if (!kBackward) {
      if (idx < n) yOut[idx] = y * net.outScale;
    } else {
      float dy = 0.0f;
      if (idx < n) {
        const float d = __ldg(samples + idx).w;
        const float target = d / net.outScale;
        const float w = fabsf(d) < band ? 10.0f : 1.0f;
        const float r = y - target;
        dy = 2.0f * w * r * invB;
        atomicAdd(loss, w * r * r * invB);
      }
      dyv[s] = dy;
    }
  }
  if (!kBackward) return;
  __syncthreads();
  for (int k = t; k < H; k += blockDim.x) {
    float acc = 0.0f;
    for (int s = 0; s < S; ++s) acc = fmaf(dyv[s], AL[s * H + k], acc);
    atomicAdd(grad + ly.wo + k, acc);
  }
  if (t == 0) {
    float acc = 0.0f;
    for (int s = 0; s < S; ++s) acc += dyv[s];
    atomicAdd(grad + ly.bo, acc);
  }
  for (int e = t; e < S * H; e += blockDim.x) {
    const int s = e / H, k = e % H;
    D0[e] = dyv[s] * __ldg(net.p + ly.wo + k) * dsilu(Z[(L - 1) * S * H + e]);
  }
  __syncthreads();
  float *cur = D0, *nxt = D1;
  for (int l = L - 1; l >= 1; --l) {
    weightGrad<H>(cur, A + (l - 1) * S * H, H, H, S, grad + ly.wh[l - 1], grad + ly.bh[l - 1]);
    // nxt[s][k] = sum_j cur[s][j] W[j][k]: W row-major is the transposed operand
    gemmTile<H>(cur, H, H, net.p + ly.wh[l - 1], nullptr, nxt);
    __syncthreads();
    for (int e = t; e < S * H; e += blockDim.x) nxt[e] *= dsilu(Z[(l - 1) * S * H + e]);
    __syncthreads();
    float *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  weightGrad<H>(cur, X, kSdfMaxInputs, D, S, grad + ly.w0, grad + ly.b0);
}

// Adam step over all parameters, then the transposed copy of every weight.
__global__ void __launch_bounds__(256)
kSdfAdam(SdfLayout ly, float *__restrict__ p, float *__restrict__ pT,
         const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v, float lr,
         float b1, float b2, float eps, float c1, float c2) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ly.total) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  unsigned j = i;  // transposed position
  if (i >= ly.w0 && i < ly.w0 + (unsigned)(ly.H * ly.D)) {
    const unsigned r = i - ly.w0;
    j = ly.w0 + (r % ly.D) * ly.H + r / ly.D;
  }
  for (int l = 1; l < ly.L; ++l) {
    const unsigned w = ly.wh[l - 1];
    if (i >= w && i < w + (unsigned)(ly.H * ly.H)) {
      const unsigned r = i - w;
      j = w + (r % ly.H) * ly.H + r / ly.H;
    }
  }
  pT[j] = pi;
}

// ---------------------------------------------------------------------------
// Tensor-core inference.
//
// Operand tiles in shared memory, K-major, no swizzle: 8-row x 16-byte core
// matrices; element (row r, k) of a tile with R rows at byte
//   (k / 8) * (R * 16) + r * 16 + (k % 8) * 2,
// so the core matrices adjacent in K are R * 16 bytes apart (the descriptor's
// leading byte offset) and those adjacent in rows 128 bytes apart (its stride
// byte offset).  A: R = 128 points; B: R = H outputs of a hidden layer.
// The accumulator D[m][n] (FP32) sits in TMEM lane m, column n.

__host__ __device__ constexpr unsigned tileOffset(int r, int k, int R) {
  return (unsigned)((k / 8) * (R * 8) + r * 8 + (k % 8));  // in bf16 elements
}

__device__ __forceinline__ unsigned smemU32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ unsigned long long umDesc(unsigned addr, unsigned lbo,
                                                     unsigned sbo) {
  return (unsigned long long)((addr & 0x3FFFFu) >> 4) |
         ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, shape M x N.
__host__ __device__ constexpr unsigned umIdesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) |
         ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void tmemAlloc(unsigned dstSmem, unsigned cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dstSmem),
               "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tmemRelinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(unsigned taddr, unsigned cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tcFenceBefore() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tcFenceAfter() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void proxyFence() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void umma(unsigned dTmem, unsigned long long a, unsigned long long b,
                                     unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void ummaCommit(unsigned mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}
__device__ __forceinline__ void mbarInit1(unsigned mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ bool mbarWaitParity(unsigned mbar, unsigned parity) {
  for (unsigned k = 0; k < kSdfWaitLimit; ++k) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmemLoad16(unsigned taddr, float (&r)[16]) {
  unsigned u[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]),
        "=r"(u[7]), "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]),
        "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int c = 0; c < 16; ++c) r[c] = __uint_as_float(u[c]);
}
__device__ __forceinline__ void tmemWaitLoad() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned packBf16(float a, float b) {
  const __nv_bfloat16 x = __float2bfloat16_rn(a), y = __float2bfloat16_rn(b);
  return (unsigned)__bfloat16_as_ushort(x) | ((unsigned)__bfloat16_as_ushort(y) << 16);
}

template <int H, int L, int T = 1>
struct SdfTileSmem {
  static_assert(H == 64 || H == 128, "width");
  static_assert(L >= 2 && L <= 3, "hidden layers");
  static_assert(T == 1 || T == 2, "tiles per CTA");
  __nv_bfloat16 a[T * 128 * H];        // activation tiles (A operands), 128 points each
  __nv_bfloat16 w[(L - 1) * H * H];    // hidden-layer weights (B operands)
  float w0[H * kSdfMaxInputs];         // first layer, [H][D]
  float b[L * H];                      // biases of the hidden layers
  float wo[H];
  float bo;
  unsigned tmem;
  unsigned long long bar;
};

// Per-CTA set-up of the tile forward: TMEM columns (H per tile), the
// barrier, the weights.  All threads of the CTA.
template <int H, int L, int T = 1>
__device__ __forceinline__ void sdfTileSetup(SdfTileSmem<H, L, T> &sm, const SdfView &net) {
  const int t = threadIdx.x;
  if (t < 32) {
    tmemAlloc(smemU32(&sm.tmem), H * T);
    tmemRelinquish();
  }
  if (t == 0) {
    mbarInit1(smemU32(&sm.bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const uint4 *src = reinterpret_cast<const uint4 *>(net.w16);
  uint4 *dst = reinterpret_cast<uint4 *>(sm.w);
  for (int e = t; e < (L - 1) * H * H / 8; e += blockDim.x) dst[e] = __ldg(src + e);
  const SdfLayout &ly = net.lay;
  for (int e = t; e < H * ly.D; e += blockDim.x) sm.w0[e] = __ldg(net.p + ly.w0 + e);
  for (int e = t; e < H; e += blockDim.x) {
    sm.b[e] = __ldg(net.p + ly.b0 + e);
    for (int l = 1; l < L; ++l) sm.b[l * H + e] = __ldg(net.p + ly.bh[l - 1] + e);
    sm.wo[e] = __ldg(net.p + ly.wo + e);
  }
  if (t == 0) sm.bo = __ldg(net.p + ly.bo);
  proxyFence();
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
}

template <int H, int L, int T = 1>
__device__ __forceinline__ void sdfTileTeardown(SdfTileSmem<H, L, T> &sm) {
  tcFenceBefore();
  __syncthreads();
  if (threadIdx.x < 32) {
    tcFenceAfter();
    tmemDealloc(sm.tmem, H * T);
  }
}

// The distance prediction for this thread's point (x normalised, shape code
// `shape` or -1); 128 * T threads, one point each, all threads of the CTA.
// Thread t works on tile t / 128, row t % 128: the tile's A operand is its
// own 128-row block of sm.a and its accumulator TMEM columns tile * H ..,
// read by the warp's lane quarter (warp % 4).  Every tile's chain uses the
// same B operands and one commit.  `phase` is the barrier parity, flipped
// per layer.  Returns false (for every thread) when an MMA chain did not
// complete in time.
template <int H, int L, int kLdBatch = 1, int T = 1>
__device__ __forceinline__ bool sdfTileForward(SdfTileSmem<H, L, T> &sm, const SdfView &net,
                                               float x0, float x1, float x2, int shape,
                                               unsigned &phase, float &dOut) {
  const int t = threadIdx.x, warp = t >> 5;
  const int tile = t >> 7, row = t & 127, quarter = warp & 3;
  __nv_bfloat16 *aTile = sm.a + tile * 128 * H;
  const int D = net.lay.D;
  // first layer on the CUDA cores, 8 outputs per 16-byte chunk of the A row
#pragma unroll 1
  for (int c = 0; c < H / 8; ++c) {
    float h[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = c * 8 + u;
      const float *w = sm.w0 + j * D;
      float z = sm.b[j];
      z = fmaf(w[0], x0, z);
      z = fmaf(w[1], x1, z);
      z = fmaf(w[2], x2, z);
      if (shape >= 0 && 3 + shape < D) z += w[3 + shape];
      h[u] = siluFast(z);
    }
    uint4 v = make_uint4(packBf16(h[0], h[1]), packBf16(h[2], h[3]), packBf16(h[4], h[5]),
                         packBf16(h[6], h[7]));
    *reinterpret_cast<uint4 *>(aTile + tileOffset(row, c * 8, 128)) = v;
  }
  proxyFence();
  tcFenceBefore();
  __syncthreads();
  const unsigned idesc = umIdesc(128, H);
  const unsigned aBase = smemU32(sm.a);
  float y = sm.bo;
  bool ok = true;
#pragma unroll 1
  for (int l = 1; l < L; ++l) {
    if (t == 0) {
      tcFenceAfter();
      const unsigned bBase = smemU32(sm.w + (l - 1) * H * H);
#pragma unroll
      for (int tt = 0; tt < T; ++tt) {
        const unsigned aTileBase = aBase + (unsigned)(tt * 128 * H * 2);
#pragma unroll
        for (int s = 0; s < H / 16; ++s)
          umma(sm.tmem + (unsigned)(tt * H), umDesc(aTileBase + s * 2 * 128 * 16, 128 * 16, 128),
               umDesc(bBase + s * 2 * H * 16, H * 16, 128), idesc, s > 0 ? 1u : 0u);
      }
      ummaCommit(smemU32(&sm.bar));
    }
    const bool done = mbarWaitParity(smemU32(&sm.bar), phase);
    phase ^= 1u;
    if (__syncthreads_or(!done)) {
      // let the chain finish (bounded) before the tile buffers are reused
      mbarWaitParity(smemU32(&sm.bar), phase ^ 1u);
      ok = false;
      break;
    }
    tcFenceAfter();
    const bool last = (l == L - 1);
    // kLdBatch column chunks of 16 are read from TMEM before one wait (more
    // loads in flight, more registers: the standalone inference kernel uses
    // 4, the fused culling kernels, which hold a particle's state, 1)
    static_assert((H / 16) % kLdBatch == 0, "column chunks per batch");
#pragma unroll 1
    for (int c0 = 0; c0 < H / 16; c0 += kLdBatch) {
      float r[kLdBatch][16];
#pragma unroll
      for (int q = 0; q < kLdBatch; ++q)
        tmemLoad16(sm.tmem + ((unsigned)(32 * quarter) << 16) +
                       (unsigned)(tile * H + (c0 + q) * 16),
                   r[q]);
      tmemWaitLoad();
#pragma unroll
      for (int q = 0; q < kLdBatch; ++q) {
        const int c = c0 + q;
#pragma unroll
        for (int u = 0; u < 16; ++u) r[q][u] = siluFast(r[q][u] + sm.b[l * H + c * 16 + u]);
        if (last) {
#pragma unroll
          for (int u = 0; u < 16; ++u) y = fmaf(r[q][u], sm.wo[c * 16 + u], y);
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            uint4 v = make_uint4(packBf16(r[q][8 * h], r[q][8 * h + 1]),
                                 packBf16(r[q][8 * h + 2], r[q][8 * h + 3]),
                                 packBf16(r[q][8 * h + 4], r[q][8 * h + 5]),
                                 packBf16(r[q][8 * h + 6], r[q][8 * h + 7]));
            *reinterpret_cast<uint4 *>(aTile + tileOffset(row, c * 16 + 8 * h, 128)) = v;
          }
        }
      }
    }
    tcFenceBefore();
    if (!last) proxyFence();
    __syncthreads();
  }
  dOut = y * net.outScale;
  return ok;
}

// d[i] for point i (float4, w ignored) with shape code shapes[i] (or none).
// kInferTiles 128-point tiles per CTA share the weights and one barrier
// round per layer; inferLd<H>() TMEM column loads are in flight per wait.
constexpr int kInferTiles = 2;
template <int H> constexpr int inferLd() { return H == 64 ? 2 : 4; }
template <int H, int L>
__global__ void __launch_bounds__(128 * kInferTiles)
kSdfInfer(SdfView net, const float4 *__restrict__ pts, const int *__restrict__ shapes,
          unsigned n, float *__restrict__ dOut, unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  SdfTileSmem<H, L, kInferTiles> &sm =
      *reinterpret_cast<SdfTileSmem<H, L, kInferTiles> *>(smraw);
  sdfTileSetup<H, L, kInferTiles>(sm, net);
  unsigned phase = 0;
  const unsigned groups = (n + 128u * kInferTiles - 1) / (128u * kInferTiles);
  for (unsigned g = blockIdx.x; g < groups; g += gridDim.x) {
    const unsigned i = g * 128u * kInferTiles + threadIdx.x;
    const bool valid = i < n;
    const float4 q = valid ? __ldg(pts + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int shape = (valid && shapes) ? __ldg(shapes + i) : -1;
    float d = 0.0f;
    if (!sdfTileForward<H, L, inferLd<H>(), kInferTiles>(
            sm, net, (q.x - net.shift[0]) * net.scale[0], (q.y - net.shift[1]) * net.scale[1],
            (q.z - net.shift[2]) * net.scale[2], shape, phase, d)) {
      if (threadIdx.x == 0) atomicOr(status, (unsigned)kStatusTimeout);
      break;
    }
    if (valid) dOut[i] = d;
  }
  sdfTileTeardown<H, L, kInferTiles>(sm);
}

// Per-tile hints of the culling kernels (performance only: results never
// depend on them).  h[tile] = 1 when, the last time the network ran on the
// tile, more than half of its in-box particles still needed the exact query;
// such a tile then queries the map directly, without the network, until a
// refresh step (every kHintRefresh steps) runs the network on every tile
// again.  h == nullptr: the network runs on every tile with a particle in
// the map box.
constexpr unsigned kHintRefresh = 8;
struct TileHints {
  unsigned char *h;
  int refresh;
};

// Culling per tile (fcdemSdfSetTileCulling).  The network runs once per
// tile of kCullTile consecutive slots, at the centre c of the box that
// bounds the tile's particles in the map box (after this step's velocity
// and position update), and the tile's exact queries are skipped when
// pred(c) - lip * rho > skin, rho being the distance from c to the box's
// corners.  With lip a Lipschitz bound of the network's prediction, every
// particle p of such a tile has pred(p) >= pred(c) - lip * |p - c| > skin:
// the per-particle rule would have skipped it as well.  Where the rule
// does not cull, every particle of the tile in the map box is queried.  A
// tile whose particles in the map box belong to scenes of different
// obstacles is not culled.
constexpr unsigned kCullTile = 32;
struct TileCull {
  const float4 *centre;  // per tile: c (x, y, z) and rho (w)
  const int *shape;      // per tile: the obstacle's shape code; -1 none in the box, -2 mixed
  const float *pred;     // per tile: the network's distance at c
  float lip, skin;
  __device__ __forceinline__ bool cull(unsigned tile) const {
    return __ldg(shape + tile) >= 0 &&
           __ldg(pred + tile) - lip * __ldg(&centre[tile].w) > skin;
  }
};

// One warp per tile: the bounding box of the tile's advanced positions in
// the map box (umAdvance: the arithmetic of the integrate that follows).
// kBatch: slot i belongs to scene sceneOf[i] with its own parameters and
// obstacle; otherwise every particle has kp and the map M.
template <bool kBatch>
__global__ void __launch_bounds__(256)
kTileCentres(const BatchScene *__restrict__ scenes, const unsigned *__restrict__ sceneOf,
             const MapView *__restrict__ maps, KParams kp, MapView M,
             const float4 *__restrict__ pos, const float4 *__restrict__ vel, float dt,
             unsigned n, float4 *__restrict__ centre, int *__restrict__ shapeOut) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned tiles = (n + kCullTile - 1) / kCullTile;
  if (tile >= tiles) return;  // whole warps leave together
  const unsigned i = tile * kCullTile + lane;
  bool in = false;
  int shape = -1;
  float3 p = make_float3(0.0f, 0.0f, 0.0f);
  if (i < n) {
    const float4 p4 = __ldg(pos + i), v4 = __ldg(vel + i);
    p = make_float3(p4.x, p4.y, p4.z);
    float3 v = make_float3(v4.x, v4.y, v4.z);
    if (kBatch) {
      const BatchScene &S = scenes[__ldg(sceneOf + i)];
      umAdvance(p, v, dt, S.p);
      shape = S.shape;
      in = shape >= 0 && inMapBox(maps[shape], p);
    } else {
      umAdvance(p, v, dt, kp.p);
      shape = 0;
      in = inMapBox(M, p);
    }
  }
  const float inf = __int_as_float(0x7f800000);
  float lx = in ? p.x : inf, ly = in ? p.y : inf, lz = in ? p.z : inf;
  float hx = in ? p.x : -inf, hy = in ? p.y : -inf, hz = in ? p.z : -inf;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
    ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
    lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
    hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
    hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
    hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
  }
  const int smin = __reduce_min_sync(0xffffffffu, in ? shape : 0x7fffffff);
  const int smax = __reduce_max_sync(0xffffffffu, in ? shape : -1);
  if (lane == 0) {
    if (smax < 0) {
      centre[tile] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      shapeOut[tile] = -1;
    } else {
      const float ex = hx - lx, ey = hy - ly, ez = hz - lz;
      // rho with a margin for the roundings of the centre and of the root
      const float rho = 0.5f * sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f + 1e-6f;
      centre[tile] = make_float4(0.5f * (lx + hx), 0.5f * (ly + hy), 0.5f * (lz + hz), rho);
      shapeOut[tile] = smin == smax ? smin : -2;
    }
  }
}

// kIntegrateDistMap's step with the map query of culled tiles skipped.
template <bool kCount>
__global__ void __launch_bounds__(256)
kIntegrateTileCull(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt, unsigned n,
                   KParams kp, MapView M, TileCull tc, unsigned *exact,
                   unsigned *__restrict__ hashOut, unsigned *__restrict__ rankOut,
                   unsigned *__restrict__ cnt, unsigned *__restrict__ tileCnt) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SimParams &P = kp.p;
  const float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  const float r = kp.radiusFromW ? p4.w : P.particleRadius;
  umAdvance(p, v, dt, P);
  const bool test = inMapBox(M, p) && !tc.cull(i / kCullTile);
  if (test && exact) atomicAdd(exact, 1u);
  umBoundary(M, test, r, P.boundaryDamping, p, v);
  if (kCount) {  // the next step's calcHash and cell count
    const int3 gp = gridPos(p.x, p.y, p.z, P);
    const unsigned h = gridHash(gp.x, gp.y, gp.z, P);
    hashOut[i] = h;
    rankOut[i] = atomicAdd(cnt + h, 1u);
    countTile(tileCnt, h >> 12);
  }
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, p4.w);
}

// d_integrateSystem + d_checkBoundaryDistMap (kIntegrateDistMap's
// arithmetic) with the map query skipped where the network predicts a
// distance above `skin`: a point outside the map box reads 5.0 from the map
// and is never tested; inside, the exact query runs only when the prediction
// is at most `skin`.  `exact` (optional) counts the exact queries.  kCount:
// also the next step's calcHash and cell count (counting-sort pipeline).
template <int H, int L, bool kCount>
__global__ void __launch_bounds__(128)
kIntegrateSdf(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt, unsigned n,
              KParams kp, MapView M, SdfView net, float skin, unsigned *exact,
              unsigned *__restrict__ hashOut, unsigned *__restrict__ rankOut,
              unsigned *__restrict__ cnt, unsigned *__restrict__ tileCnt, TileHints hints,
              unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  SdfTileSmem<H, L> &sm = *reinterpret_cast<SdfTileSmem<H, L> *>(smraw);
  sdfTileSetup<H, L>(sm, net);
  const SimParams &P = kp.p;
  unsigned phase = 0;
  const unsigned tiles = (n + 127) / 128;
  for (unsigned tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const unsigned i = tile * 128 + threadIdx.x;
    const bool valid = i < n;
    float4 p4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v4 = p4;
    if (valid) {
      p4 = pos[i];
      v4 = vel[i];
    }
    float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
    const float r = kp.radiusFromW ? p4.w : P.particleRadius;
    umAdvance(p, v, dt, P);
    const bool inBox = valid && inMapBox(M, p);
    float dPred = 0.0f;
    // a tile with no particle in the map box needs no prediction (the map
    // reads 5.0 outside its box); the decisions are the same for every thread
    const bool anyIn = __syncthreads_or(inBox);
    const bool useNet = anyIn && (!hints.h || hints.refresh || hints.h[tile] == 0);
    if (useNet &&
        !sdfTileForward<H, L>(sm, net, (p.x - net.shift[0]) * net.scale[0],
                              (p.y - net.shift[1]) * net.scale[1],
                              (p.z - net.shift[2]) * net.scale[2], 0, phase, dPred)) {
      if (threadIdx.x == 0) atomicOr(status, (unsigned)kStatusTimeout);
      break;
    }
    const bool test = inBox && (!useNet || !(dPred > skin));
    if (useNet && hints.h) {
      const int nIn = __syncthreads_count(inBox), nTest = __syncthreads_count(test);
      if (threadIdx.x == 0) hints.h[tile] = 2 * nTest > nIn ? 1 : 0;
    }
    if (!valid) continue;
    if (test && exact) atomicAdd(exact, 1u);
    umBoundary(M, test, r, P.boundaryDamping, p, v);
    if (kCount) {  // the next step's calcHash and cell count
      const int3 gp = gridPos(p.x, p.y, p.z, P);
      const unsigned h = gridHash(gp.x, gp.y, gp.z, P);
      hashOut[i] = h;
      rankOut[i] = atomicAdd(cnt + h, 1u);
      countTile(tileCnt, h >> 12);
    }
    pos[i] = make_float4(p.x, p.y, p.z, p4.w);
    vel[i] = make_float4(v.x, v.y, v.z, p4.w);
  }
  sdfTileTeardown<H, L>(sm);
}

// integrateOneBox's clamp to the scene box, same faces in the same order,
// the roundings spelled out.
__device__ __forceinline__ void boxClamp(float3 &p, float3 &v, float r, float bd,
                                         const float *lo, const float *hi) {
  if (p.x > hi[0] - r) { p.x = hi[0] - r; v.x = __fmul_rn(v.x, bd); }
  if (p.x < lo[0] + r) { p.x = lo[0] + r; v.x = __fmul_rn(v.x, bd); }
  if (p.y > hi[1] - r) { p.y = hi[1] - r; v.y = __fmul_rn(v.y, bd); }
  if (p.z > hi[2] - r) { p.z = hi[2] - r; v.z = __fmul_rn(v.z, bd); }
  if (p.z < lo[2] + r) { p.z = lo[2] + r; v.z = __fmul_rn(v.z, bd); }
  if (p.y < lo[1] + r) { p.y = lo[1] + r; v.y = __fmul_rn(v.y, bd); }
}

// Batch integrate with obstacles: particle / slot i belongs to scene
// sceneOf[i]; the velocity and position update, the contact of the scene's
// obstacle map (checkDistMap), the clamp to the scene's box, and with
// doCount the next global cell id and count.  kNet: a tile of 128 with a
// particle in its obstacle's map box runs the network (the scene's shape as
// the one-hot code) and only particles predicted within `skin` query the map.
// Without kNet, tc (when set) holds the decisions of the culling per tile.
template <int H, int L, bool kNet, bool kW>
__global__ void __launch_bounds__(128)
kBatchObstacle(const BatchScene *__restrict__ scenes, const unsigned *__restrict__ sceneOf,
               const MapView *__restrict__ maps, SdfView net, float skin,
               const float4 *__restrict__ inPos, float4 *__restrict__ pos,
               float4 *__restrict__ vel, float dt, unsigned n, UmCount count, int doCount,
               unsigned *exact, TileHints hints, TileCull tc, unsigned *status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  SdfTileSmem<H, L> &sm = *reinterpret_cast<SdfTileSmem<H, L> *>(smraw);
  if (kNet) sdfTileSetup<H, L>(sm, net);
  unsigned phase = 0;
  const unsigned tiles = (n + 127) / 128;
  for (unsigned tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const unsigned i = tile * 128 + threadIdx.x;
    const bool valid = i < n;
    const BatchScene *S = valid ? scenes + __ldg(sceneOf + i) : scenes;
    const SimParams &P = S->p;
    float4 p4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v4 = p4;
    if (valid) {
      p4 = inPos[i];
      v4 = vel[i];
    }
    float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
    const float r = kW ? p4.w : P.particleRadius;
    umAdvance(p, v, dt, P);
    const int shape = valid ? S->shape : -1;
    MapView M{};
    if (shape >= 0) M = maps[shape];
    const bool inBox = shape >= 0 && inMapBox(M, p);
    float dPred = 0.0f;
    bool useNet = false;
    if (kNet) {
      const bool anyIn = __syncthreads_or(inBox);
      useNet = anyIn && (!hints.h || hints.refresh || hints.h[tile] == 0);
      if (useNet &&
          !sdfTileForward<H, L>(sm, net, (p.x - net.shift[0]) * net.scale[0],
                                (p.y - net.shift[1]) * net.scale[1],
                                (p.z - net.shift[2]) * net.scale[2], shape, phase, dPred)) {
        if (threadIdx.x == 0) atomicOr(status, (unsigned)kStatusTimeout);
        break;
      }
    }
    // without the network in the kernel: the tiles' decisions (TileCull), if any
    const bool test = inBox && (!useNet || !(dPred > skin)) &&
                      (kNet || !tc.shape || !tc.cull(i / kCullTile));
    if (kNet && useNet && hints.h) {
      const int nIn = __syncthreads_count(inBox), nTest = __syncthreads_count(test);
      if (threadIdx.x == 0) hints.h[tile] = 2 * nTest > nIn ? 1 : 0;
    }
    if (!valid) continue;
    if (test) {
      if (exact) atomicAdd(exact, 1u);
      checkDistMap(M, r, P.boundaryDamping, p, v);
    }
    boxClamp(p, v, r, P.boundaryDamping, S->lo, S->hi);
    pos[i] = make_float4(p.x, p.y, p.z, p4.w);
    vel[i] = make_float4(v.x, v.y, v.z, v4.w);
    if (doCount) {
      const int3 gp = gridPos(p.x, p.y, p.z, P);
      const unsigned h = S->cellBase + gridHash(gp.x, gp.y, gp.z, P);
      count.hash[i] = h;
      count.rank[i] = atomicAdd(count.cnt + h, 1u);
      countTile(count.tileCnt, h >> 12);
    }
  }
  if (kNet) sdfTileTeardown<H, L>(sm);
}

// Hidden-layer weights, FP32 [out][in], to the BF16 B-operand tiles.
__global__ void __launch_bounds__(256)
kSdfPackBf16(const float *__restrict__ p, SdfLayout ly, __nv_bfloat16 *__restrict__ w16) {
  const int H = ly.H;
  const unsigned per = (unsigned)(H * H);
  const unsigned total = per * (unsigned)(ly.L - 1);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    const unsigned l = e / per, r = e % per;
    const int o = (int)(r / H), k = (int)(r % H);
    w16[l * per + tileOffset(o, k, H)] = __float2bfloat16_rn(p[ly.wh[l] + r]);
  }
}

}  // namespace
}  // namespace fcdem

using namespace fcdem;

struct fcdemSdfNet {
  int device = -1;
  SdfLayout lay{};
  float shift[3] = {0.0f, 0.0f, 0.0f}, scale[3] = {1.0f, 1.0f, 1.0f}, outScale = 1.0f;
  float *params = nullptr, *paramsT = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  float *loss = nullptr;  // one device float
  __nv_bfloat16 *w16 = nullptr;
  bool w16Fresh = false;
  unsigned adamStep = 0;
  unsigned version = 0;  // bumped whenever the weights or the normalisation change
  unsigned char *hints = nullptr;  // per-tile culling hints (TileHints)
  unsigned hintTiles = 0;
  float tileLip = 0.0f;          // > 0: cull per tile of kCullTile slots (TileCull)
  void *tileBuf = nullptr;       // TileCull's centres, shapes and predictions
  unsigned tileCap = 0;          // tiles tileBuf holds
};

namespace fcdem {
namespace {

bool shapeOk(int D, int H, int L) {
  return D >= 3 && D <= kSdfMaxInputs && (H == 64 || H == 128) && L >= 2 && L <= 3;
}

SdfView sdfView(const fcdemSdfNet *net) {
  SdfView v;
  v.lay = net->lay;
  v.p = net->params;
  v.pT = net->paramsT;
  v.w16 = net->w16;
  for (int k = 0; k < 3; ++k) {
    v.shift[k] = net->shift[k];
    v.scale[k] = net->scale[k];
  }
  v.outScale = net->outScale;
  return v;
}

void freeNet(fcdemSdfNet *net) {
  if (!net) return;
  cudaFree(net->params);
  cudaFree(net->paramsT);
  cudaFree(net->grad);
  cudaFree(net->m);
  cudaFree(net->v);
  cudaFree(net->loss);
  cudaFree(net->w16);
  cudaFree(net->hints);
  cudaFree(net->tileBuf);
  delete net;
}

std::vector<float> transposed(const SdfLayout &ly, const std::vector<float> &p) {
  std::vector<float> t(p);
  for (int j = 0; j < ly.H; ++j)
    for (int d = 0; d < ly.D; ++d) t[ly.w0 + d * ly.H + j] = p[ly.w0 + j * ly.D + d];
  for (int l = 1; l < ly.L; ++l)
    for (int j = 0; j < ly.H; ++j)
      for (int k = 0; k < ly.H; ++k)
        t[ly.wh[l - 1] + k * ly.H + j] = p[ly.wh[l - 1] + j * ly.H + k];
  return t;
}

bool uploadParams(fcdemSdfNet *net, const std::vector<float> &p) {
  const std::vector<float> t = transposed(net->lay, p);
  const size_t bytes = sizeof(float) * p.size();
  net->w16Fresh = false;
  net->version++;
  return cudaOk(cudaMemcpy(net->params, p.data(), bytes, cudaMemcpyHostToDevice)) &&
         cudaOk(cudaMemcpy(net->paramsT, t.data(), bytes, cudaMemcpyHostToDevice));
}

template <int H, int L>
size_t tileSmemBytes() {
  return sizeof(SdfTileSmem<H, L>) + 1024;  // + alignment slack
}

bool packWeights(fcdemSdfNet *net) {
  if (net->w16Fresh) return true;
  kSdfPackBf16<<<64, 256, 0, curStream()>>>(net->params, net->lay, net->w16);
  if (!launchOk()) return false;
  net->w16Fresh = true;
  return true;
}

// Runs the forward (+ backward) tile kernel over n samples.
bool runTrainKernel(fcdemSdfNet *net, bool backward, const float4 *samples, const int *shapes,
                    unsigned n, float band, float invB, float *yOut) {
  const SdfView v = sdfView(net);
  const int H = net->lay.H, L = net->lay.L;
  const unsigned S = 4096u / (unsigned)H;
  const unsigned blocks = (n + S - 1) / S;
  cudaStream_t st = curStream();
#define FCDEM_SDF_TRAIN(HH, LL)                                                              \
  if (H == HH && L == LL) {                                                                  \
    const size_t smem = trainSmemBytes<HH, LL>();                                            \
    if (backward) {                                                                          \
      cudaFuncSetAttribute(kSdfTrain<HH, LL, true>,                                          \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);          \
      kSdfTrain<HH, LL, true><<<blocks, 256, smem, st>>>(v, samples, shapes, n, band, invB,  \
                                                         net->grad, net->loss, nullptr);     \
    } else {                                                                                 \
      cudaFuncSetAttribute(kSdfTrain<HH, LL, false>,                                         \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);          \
      kSdfTrain<HH, LL, false><<<blocks, 256, smem, st>>>(v, samples, shapes, n, band, invB, \
                                                          nullptr, nullptr, yOut);           \
    }                                                                                        \
    return launchOk();                                                                       \
  }
  FCDEM_SDF_TRAIN(64, 3)
  FCDEM_SDF_TRAIN(64, 2)
  FCDEM_SDF_TRAIN(128, 2)
  FCDEM_SDF_TRAIN(128, 3)
#undef FCDEM_SDF_TRAIN
  setError(FCDEM_ERR_INVALID_VALUE);
  return false;
}

bool adamStep(fcdemSdfNet *net, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  net->adamStep++;
  net->version++;
  const double t = (double)net->adamStep;
  const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, t)));
  const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, t)));
  kSdfAdam<<<(net->lay.total + 255) / 256, 256, 0, curStream()>>>(
      net->lay, net->params, net->paramsT, net->grad, net->m, net->v, lr, b1, b2, eps, c1, c2);
  net->w16Fresh = false;
  return launchOk();
}

// CTAs per SM that fit both the shared memory (227 KB) and the 512 TMEM
// columns (H per CTA); the persistent grid is the SM count times that.
template <int H, int L>
constexpr unsigned sdfCtasPerSm() {
  constexpr unsigned bySmem = (unsigned)((227u * 1024u) / (sizeof(SdfTileSmem<H, L>) + 1024u));
  constexpr unsigned byTmem = 512u / (unsigned)H;
  return bySmem < byTmem ? bySmem : byTmem;
}

template <int H, int L>
bool launchInfer(fcdemSdfNet *net, const float4 *pts, const int *shapes, unsigned n,
                 float *d) {
  const size_t smem = sizeof(SdfTileSmem<H, L, kInferTiles>) + 1024;  // + alignment slack
  const int threads = 128 * kInferTiles;
  // persistent grid: the CTAs that are resident at once (registers, shared
  // memory), capped by the 512 TMEM columns of an SM (H per tile): a CTA
  // beyond that would wait in tcgen05.alloc for columns no CTA frees.
  // Worked out once per device (the attribute calls cost more host time
  // than a launch).
  static int residentOf[64] = {};
  int dev = 0;
  if (!cudaOk(cudaGetDevice(&dev))) return false;
  if (dev < 0 || dev >= 64) dev = 0;
  int resident = residentOf[dev];
  if (resident == 0) {
    // the whole carveout as shared memory
    if (!cudaOk(cudaFuncSetAttribute(kSdfInfer<H, L>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) ||
        !cudaOk(cudaFuncSetAttribute(kSdfInfer<H, L>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared)))
      return false;
    cudaFuncAttributes fa;
    if (!cudaOk(cudaFuncGetAttributes(&fa, kSdfInfer<H, L>))) return false;
    // registers are allocated per warp in units of 256
    const int regsPerWarp = ((fa.numRegs * 32 + 255) / 256) * 256;
    const int byRegs = regsPerWarp > 0 ? (65536 / regsPerWarp) / (threads / 32) : 1;
    const int bySmem = (int)((227u * 1024u) / (smem + 1024u));  // + the per-CTA reserve
    const int byTmem = 512 / (H * kInferTiles);
    resident = byRegs < bySmem ? byRegs : bySmem;
    if (resident > byTmem) resident = byTmem;
    if (resident < 1) resident = 1;
    residentOf[dev] = resident;
  }
  unsigned grid = (n + 128u * kInferTiles - 1) / (128u * kInferTiles);
  if (grid > numSms() * (unsigned)resident) grid = numSms() * (unsigned)resident;
  kSdfInfer<H, L><<<grid, threads, smem, curStream()>>>(sdfView(net), pts, shapes, n, d,
                                                        ctx().dStatus);
  return launchOk();
}

template <int H, int L>
bool launchIntegrateSdf(fcdemSdfNet *net, float4 *pos, float4 *vel, float dt, unsigned n,
                        const KParams &kp, const MapView &M, float skin, unsigned *exact,
                        const UmCount *count, TileHints hints) {
  const size_t smem = tileSmemBytes<H, L>();
  unsigned grid = (n + 127) / 128;
  if (grid > numSms() * sdfCtasPerSm<H, L>()) grid = numSms() * sdfCtasPerSm<H, L>();
  if (count) {
    cudaFuncSetAttribute(kIntegrateSdf<H, L, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    kIntegrateSdf<H, L, true><<<grid, 128, smem, curStream()>>>(
        pos, vel, dt, n, kp, M, sdfView(net), skin, exact, count->hash, count->rank, count->cnt,
        count->tileCnt, hints, ctx().dStatus);
  } else {
    cudaFuncSetAttribute(kIntegrateSdf<H, L, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    kIntegrateSdf<H, L, false><<<grid, 128, smem, curStream()>>>(
        pos, vel, dt, n, kp, M, sdfView(net), skin, exact, nullptr, nullptr, nullptr, nullptr,
        hints, ctx().dStatus);
  }
  return launchOk();
}

template <int H, int L, bool kNet, bool kW>
bool launchBatchObstacle(fcdemSdfNet *net, const BatchScene *scenes, const unsigned *sceneOf,
                         const MapView *maps, float skin, const float4 *inPos, float4 *pos,
                         float4 *vel, float dt, unsigned n, const UmCount *count,
                         unsigned *exact, TileHints hints, TileCull tc = TileCull{}) {
  unsigned grid = (n + 127) / 128;
  size_t smem = 0;
  SdfView v{};
  if (kNet) {
    smem = tileSmemBytes<H, L>();
    cudaFuncSetAttribute(kBatchObstacle<H, L, kNet, kW>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (grid > numSms() * sdfCtasPerSm<H, L>()) grid = numSms() * sdfCtasPerSm<H, L>();
    v = sdfView(net);
  }
  kBatchObstacle<H, L, kNet, kW><<<grid, 128, smem, curStream()>>>(
      scenes, sceneOf, maps, v, skin, inPos, pos, vel, dt, n, count ? *count : UmCount{},
      count ? 1 : 0, exact, hints, tc, ctx().dStatus);
  return launchOk();
}

}  // namespace
}  // namespace fcdem

namespace fcdem {

unsigned sdfVersion(const fcdemSdfNet *net) { return net ? net->version : 0u; }

// The net's hint array for `tiles` tiles (grown on demand, cleared when
// grown); nullptr (no hints) when it cannot be had.
unsigned char *sdfHints(fcdemSdfNet *net, unsigned tiles) {
  if (net->hints && net->hintTiles >= tiles) return net->hints;
  if (!cudaOk(cudaDeviceSynchronize())) return nullptr;
  cudaFree(net->hints);
  net->hints = nullptr;
  net->hintTiles = 0;
  if (cudaMalloc(&net->hints, tiles) != cudaSuccess) {
    cudaGetLastError();
    net->hints = nullptr;
    return nullptr;
  }
  if (!cudaOk(cudaMemset(net->hints, 0, tiles))) return nullptr;
  net->hintTiles = tiles;
  return net->hints;
}

// The net's per-tile arrays of the culling per tile, for n slots (grown on
// demand); nullptr when they cannot be had.
bool sdfTileBuffers(fcdemSdfNet *net, unsigned n, TileCull &tc) {
  const unsigned tiles = (n + kCullTile - 1) / kCullTile;
  if (!net->tileBuf || net->tileCap < tiles) {
    if (!cudaOk(cudaDeviceSynchronize())) return false;
    cudaFree(net->tileBuf);
    net->tileBuf = nullptr;
    net->tileCap = 0;
    if (cudaMalloc(&net->tileBuf, (size_t)tiles * 24) != cudaSuccess) {
      cudaGetLastError();
      setError(FCDEM_ERR_ALLOC);
      return false;
    }
    net->tileCap = tiles;
  }
  float4 *centre = (float4 *)net->tileBuf;
  int *shape = (int *)(centre + net->tileCap);
  float *pred = (float *)(shape + net->tileCap);
  tc = TileCull{centre, shape, pred, net->tileLip, 0.0f};
  return true;
}

bool sdfPrepareTiles(fcdemSdfNet *net, unsigned n) {
  TileCull tc{};
  return !net || !(net->tileLip > 0.0f) || n == 0 || sdfTileBuffers(net, n, tc);
}

// The tiles' centres and the network's predictions there (culling per tile).
template <bool kBatch>
bool tileDecisions(fcdemSdfNet *net, const BatchScene *scenes, const unsigned *sceneOf,
                   const MapView *maps, const KParams &kp, const MapView &M,
                   const float4 *inPos, const float4 *vel, float dt, unsigned n, float skin,
                   TileCull &tc) {
  if (!sdfTileBuffers(net, n, tc)) return false;
  tc.skin = skin;
  const unsigned tiles = (n + kCullTile - 1) / kCullTile;
  kTileCentres<kBatch><<<(tiles * 32 + 255) / 256, 256, 0, curStream()>>>(
      scenes, sceneOf, maps, kp, M, inPos, vel, dt, n, const_cast<float4 *>(tc.centre),
      const_cast<int *>(tc.shape));
  if (!launchOk()) return false;
  // the shape codes go to the network too (a negative code: no one-hot input)
  const int *shapes = kBatch ? tc.shape : nullptr;
  const int H = net->lay.H, L = net->lay.L;
  float *pred = const_cast<float *>(tc.pred);
  if (H == 64 && L == 3) return launchInfer<64, 3>(net, tc.centre, shapes, tiles, pred);
  if (H == 64 && L == 2) return launchInfer<64, 2>(net, tc.centre, shapes, tiles, pred);
  if (H == 128 && L == 2) return launchInfer<128, 2>(net, tc.centre, shapes, tiles, pred);
  if (H == 128 && L == 3) return launchInfer<128, 3>(net, tc.centre, shapes, tiles, pred);
  setError(FCDEM_ERR_INVALID_VALUE);
  return false;
}

bool batchObstacleIntegrate(const BatchScene *scenes, const unsigned *sceneOf, bool radiusFromW,
                            const MapView *maps, fcdemSdfNet *net, float skin,
                            const float4 *inPos, float4 *pos, float4 *vel, float dt,
                            unsigned n, const UmCount *count, unsigned *exact, unsigned step) {
  if (n == 0) return true;
  if (net && net->tileLip > 0.0f) {
    if (!packWeights(net)) return false;
    TileCull tc{};
    if (!tileDecisions<true>(net, scenes, sceneOf, maps, KParams{}, MapView{}, inPos, vel, dt,
                             n, skin, tc))
      return false;
    const TileHints none{nullptr, 1};
    return radiusFromW
               ? launchBatchObstacle<64, 3, false, true>(net, scenes, sceneOf, maps, skin, inPos,
                                                         pos, vel, dt, n, count, exact, none, tc)
               : launchBatchObstacle<64, 3, false, false>(net, scenes, sceneOf, maps, skin,
                                                          inPos, pos, vel, dt, n, count, exact,
                                                          none, tc);
  }
  if (!net) {
    const TileHints none{nullptr, 1};
    return radiusFromW
               ? launchBatchObstacle<64, 3, false, true>(net, scenes, sceneOf, maps, skin, inPos,
                                                         pos, vel, dt, n, count, exact, none)
               : launchBatchObstacle<64, 3, false, false>(net, scenes, sceneOf, maps, skin,
                                                          inPos, pos, vel, dt, n, count, exact,
                                                          none);
  }
  if (!packWeights(net)) return false;
  const TileHints hints{sdfHints(net, (n + 127) / 128), step % kHintRefresh == 0 ? 1 : 0};
  const int H = net->lay.H, L = net->lay.L;
#define FCDEM_BATCH_OBST(HH, LL)                                                             \
  if (H == HH && L == LL)                                                                    \
    return radiusFromW ? launchBatchObstacle<HH, LL, true, true>(net, scenes, sceneOf, maps, \
                                                                 skin, inPos, pos, vel, dt,  \
                                                                 n, count, exact, hints)     \
                       : launchBatchObstacle<HH, LL, true, false>(                           \
                             net, scenes, sceneOf, maps, skin, inPos, pos, vel, dt, n,       \
                             count, exact, hints);
  FCDEM_BATCH_OBST(64, 3)
  FCDEM_BATCH_OBST(64, 2)
  FCDEM_BATCH_OBST(128, 2)
  FCDEM_BATCH_OBST(128, 3)
#undef FCDEM_BATCH_OBST
  setError(FCDEM_ERR_INVALID_VALUE);
  return false;
}

bool sdfIntegrate(fcdemSdfNet *net, float4 *pos, float4 *vel, float dt, unsigned n,
                  const KParams &kp, const fcdemDistanceMap *map, float skin, unsigned *exact,
                  const UmCount *count, int step) {
  if (!packWeights(net)) return false;
  const int H = net->lay.H, L = net->lay.L;
  const MapView M = view(map);
  if (net->tileLip > 0.0f) {
    if (n == 0) return true;
    TileCull tc{};
    if (!tileDecisions<false>(net, nullptr, nullptr, nullptr, kp, M, pos, vel, dt, n, skin, tc))
      return false;
    const unsigned blocks = (n + 255) / 256;
    if (count)
      kIntegrateTileCull<true><<<blocks, 256, 0, curStream()>>>(
          pos, vel, dt, n, kp, M, tc, exact, count->hash, count->rank, count->cnt,
          count->tileCnt);
    else
      kIntegrateTileCull<false><<<blocks, 256, 0, curStream()>>>(
          pos, vel, dt, n, kp, M, tc, exact, nullptr, nullptr, nullptr, nullptr);
    return launchOk();
  }
  // step < 0: a lone call, no hints
  const TileHints hints{step < 0 ? nullptr : sdfHints(net, (n + 127) / 128),
                        (step < 0 || step % (int)kHintRefresh == 0) ? 1 : 0};
  if (H == 64 && L == 3) return launchIntegrateSdf<64, 3>(net, pos, vel, dt, n, kp, M, skin, exact, count, hints);
  if (H == 64 && L == 2) return launchIntegrateSdf<64, 2>(net, pos, vel, dt, n, kp, M, skin, exact, count, hints);
  if (H == 128 && L == 2) return launchIntegrateSdf<128, 2>(net, pos, vel, dt, n, kp, M, skin, exact, count, hints);
  if (H == 128 && L == 3) return launchIntegrateSdf<128, 3>(net, pos, vel, dt, n, kp, M, skin, exact, count, hints);
  setError(FCDEM_ERR_INVALID_VALUE);
  return false;
}

}  // namespace fcdem

extern "C" {

fcdemSdfNet *fcdemSdfCreate(int inputs, int hidden, int hiddenLayers, unsigned long long seed) {
  if (!shapeOk(inputs, hidden, hiddenLayers)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return nullptr;
  }
  ctx();
  fcdemSdfNet *net = new fcdemSdfNet();
  cudaGetDevice(&net->device);
  net->lay = makeLayout(inputs, hidden, hiddenLayers);
  const size_t bytes = sizeof(float) * net->lay.total;
  const size_t w16 = sizeof(__nv_bfloat16) * (size_t)(hiddenLayers - 1) * hidden * hidden;
  bool ok = cudaMalloc(&net->params, bytes) == cudaSuccess &&
            cudaMalloc(&net->paramsT, bytes) == cudaSuccess &&
            cudaMalloc(&net->grad, bytes) == cudaSuccess &&
            cudaMalloc(&net->m, bytes) == cudaSuccess && cudaMalloc(&net->v, bytes) == cudaSuccess &&
            cudaMalloc(&net->loss, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&net->w16, w16) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    setError(FCDEM_ERR_ALLOC);
    freeNet(net);
    return nullptr;
  }
  // uniform initialisation, bound sqrt(6 / fan_in) (weights), zero biases
  std::vector<float> p(net->lay.total, 0.0f);
  unsigned long long z = seed;
  auto next = [&z]() {
    z += 0x9e3779b97f4a7c15ull;
    unsigned long long x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  const SdfLayout &ly = net->lay;
  auto fill = [&](unsigned off, unsigned count, int fanIn) {
    const double bound = std::sqrt(6.0 / (double)fanIn);
    for (unsigned k = 0; k < count; ++k) p[off + k] = (float)((2.0 * next() - 1.0) * bound);
  };
  fill(ly.w0, (unsigned)(ly.H * ly.D), 3);
  for (int l = 1; l < ly.L; ++l) fill(ly.wh[l - 1], (unsigned)(ly.H * ly.H), ly.H);
  fill(ly.wo, (unsigned)ly.H, ly.H);
  if (!uploadParams(net, p) || !cudaOk(cudaMemset(net->m, 0, bytes)) ||
      !cudaOk(cudaMemset(net->v, 0, bytes))) {
    freeNet(net);
    return nullptr;
  }
  return net;
}

void fcdemSdfDestroy(fcdemSdfNet *net) { freeNet(net); }

uint fcdemSdfNumParams(const fcdemSdfNet *net) { return net ? net->lay.total : 0u; }

void fcdemSdfGetParams(const fcdemSdfNet *net, float *host) {
  if (!net || !host) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  cudaOk(cudaMemcpy(host, net->params, sizeof(float) * net->lay.total, cudaMemcpyDeviceToHost));
}

void fcdemSdfSetParams(fcdemSdfNet *net, const float *host) {
  if (!net || !host) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  std::vector<float> p(host, host + net->lay.total);
  uploadParams(net, p);
}

void fcdemSdfSetNormalization(fcdemSdfNet *net, const float shift[3], const float scale[3],
                              float outScale) {
  if (!net || !shift || !scale || !(outScale > 0.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  for (int k = 0; k < 3; ++k) {
    net->shift[k] = shift[k];
    net->scale[k] = scale[k];
  }
  net->outScale = outScale;
  net->version++;
}

void fcdemSdfSetTileCulling(fcdemSdfNet *net, float lipschitz) {
  if (!net || !(lipschitz >= 0.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  net->tileLip = lipschitz;
  net->version++;  // a recorded batch graph holds the launches of the other mode
}

void fcdemSdfGetNormalization(const fcdemSdfNet *net, float shift[3], float scale[3],
                              float *outScale) {
  if (!net) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  for (int k = 0; k < 3; ++k) {
    if (shift) shift[k] = net->shift[k];
    if (scale) scale[k] = net->scale[k];
  }
  if (outScale) *outScale = net->outScale;
}

void fcdemSdfSamples(const fcdemDistanceMap *map, int shape, uint n, float nearFraction,
                     float band, unsigned long long seed, float *samples4, int *shapes) {
  if (!map || (n && !samples4) || !(nearFraction >= 0.0f && nearFraction <= 1.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  if (n == 0) return;
  const unsigned nNear = (unsigned)((double)n * nearFraction);
  kSdfSamples<<<(n + 255) / 256, 256, 0, curStream()>>>(view(map), (float4 *)samples4, shapes,
                                                        shape, n, nNear, band, seed);
  launchOk();
}

float fcdemSdfGradient(fcdemSdfNet *net, const float *samples4, const int *shapes, uint n,
                       float band, float *gradHost) {
  if (!net || !samples4 || n == 0) { setError(FCDEM_ERR_INVALID_VALUE); return 0.0f; }
  const size_t bytes = sizeof(float) * net->lay.total;
  if (!cudaOk(cudaMemsetAsync(net->grad, 0, bytes, curStream())) ||
      !cudaOk(cudaMemsetAsync(net->loss, 0, sizeof(float), curStream())))
    return 0.0f;
  if (!runTrainKernel(net, true, (const float4 *)samples4, shapes, n, band, 1.0f / (float)n,
                      nullptr))
    return 0.0f;
  float loss = 0.0f;
  cudaOk(cudaStreamSynchronize(curStream()));
  cudaOk(cudaMemcpy(&loss, net->loss, sizeof(float), cudaMemcpyDeviceToHost));
  if (gradHost) cudaOk(cudaMemcpy(gradHost, net->grad, bytes, cudaMemcpyDeviceToHost));
  return loss;
}

float fcdemSdfTrainSamples(fcdemSdfNet *net, const float *samples4, const int *shapes, uint n,
                           uint epochs, uint batch, float lr, float band) {
  if (!net || !samples4 || n == 0 || batch == 0 || epochs == 0) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return 0.0f;
  }
  const size_t bytes = sizeof(float) * net->lay.total;
  const unsigned batches = (n + batch - 1) / batch;
  const unsigned total = batches * epochs;
  float last = 0.0f;
  for (unsigned e = 0; e < epochs; ++e) {
    if (!cudaOk(cudaMemsetAsync(net->loss, 0, sizeof(float), curStream()))) return 0.0f;
    for (unsigned b = 0; b < batches; ++b) {
      const unsigned off = b * batch;
      const unsigned cnt = (n - off) < batch ? (n - off) : batch;
      // cosine decay to lr / 20 over the whole run
      const double prog = (double)(e * batches + b) / (double)total;
      const float lrNow =
          (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.14159265358979 * prog))));
      if (!cudaOk(cudaMemsetAsync(net->grad, 0, bytes, curStream()))) return 0.0f;
      if (!runTrainKernel(net, true, (const float4 *)samples4 + off, shapes ? shapes + off : nullptr,
                          cnt, band, 1.0f / (float)cnt, nullptr))
        return 0.0f;
      if (!adamStep(net, lrNow)) return 0.0f;
    }
    if (e + 1 == epochs) {
      cudaOk(cudaStreamSynchronize(curStream()));
      cudaOk(cudaMemcpy(&last, net->loss, sizeof(float), cudaMemcpyDeviceToHost));
      last /= (float)batches;
    }
  }
  return last;
}

void fcdemSdfEvalF32(fcdemSdfNet *net, const float *points4, const int *shapes, uint n,
                     float *d) {
  if (!net || (n && (!points4 || !d))) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (n == 0) return;
  runTrainKernel(net, false, (const float4 *)points4, shapes, n, 0.0f, 0.0f, d);
}

void fcdemSdfInfer(fcdemSdfNet *net, const float *points4, const int *shapes, uint n,
                   float *d) {
  if (!net || (n && (!points4 || !d))) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (n == 0) return;
  if (!packWeights(net)) return;
  const int H = net->lay.H, L = net->lay.L;
  if (H == 64 && L == 3) launchInfer<64, 3>(net, (const float4 *)points4, shapes, n, d);
  else if (H == 64 && L == 2) launchInfer<64, 2>(net, (const float4 *)points4, shapes, n, d);
  else if (H == 128 && L == 2) launchInfer<128, 2>(net, (const float4 *)points4, shapes, n, d);
  else if (H == 128 && L == 3) launchInfer<128, 3>(net, (const float4 *)points4, shapes, n, d);
  else setError(FCDEM_ERR_INVALID_VALUE);
}

void fcdemUM_integrateSystemSdf(float *pos, float *vel, float deltaTime, uint numParticles,
                                const fcdemDistanceMap *map, fcdemSdfNet *net, float skin,
                                uint *exactQueries) {
  Context &c = ctx();
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return; }
  if (numParticles == 0) return;
  if (!pos || !vel || !map || !net || !(skin >= 0.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  sdfIntegrate(net, (float4 *)pos, (float4 *)vel, deltaTime, numParticles, kparams(c), map, skin,
               exactQueries, nullptr, -1);
}

}  // extern "C"
