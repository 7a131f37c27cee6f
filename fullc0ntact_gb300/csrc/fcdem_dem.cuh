// fcdem_dem.cuh -- per-particle device arithmetic of the DEM step.
//
// Each function states the reference routine it reproduces, with the same
// operations in the same order.  Where the reference's CUDA code leaves nvcc
// to contract `a * b + c` into a fused multiply-add, the contraction is
// written out here (fmaf, __fmul_rn, __fadd_rn): every kernel that inlines
// these functions computes the same bits, and a CPU restatement with the
// same fmaf calls reproduces them exactly.
#pragma once

#include "fcdem_internal.cuh"

namespace fcdem {

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// particles_kernel.cu:78-85 (calcGridPos): IEEE division and floor, then the
// float->int conversion of the assignment.
__device__ __forceinline__ int3 gridPos(float px, float py, float pz,
                                        const SimParams &P) {
  int3 g;
  g.x = (int)floorf((px - P.worldOrigin[0]) / P.cellSize[0]);
  g.y = (int)floorf((py - P.worldOrigin[1]) / P.cellSize[1]);
  g.z = (int)floorf((pz - P.worldOrigin[2]) / P.cellSize[2]);
  return g;
}

// Cell-key order.  The library's own copy of SimParams carries kMortonTag in
// maxParticlesPerCell (a field the reference never reads) when
// fcdemSetCellOrder(1) is on and the grid is cubic: every cell key is then
// the Morton code of the wrapped cell coordinates instead of the linear
// hash.  Morton order keeps cells that are near in space near in the sorted
// arrays; the per-cell contents and their order are the same either way.
// Bits 0..9 of v moved to bits 0, 3, 6, ... 27 (3-D Morton spread).
__device__ __forceinline__ unsigned mortonSpread(unsigned v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ bool mortonOrder(const SimParams &P) {
  return P.maxParticlesPerCell == kMortonTag;
}

// particles_kernel.cu:88-94 (calcGridHash): power-of-two wrap, 24-bit
// multiplies -- or, in Morton order, the interleaved bits of the wrapped
// coordinates (x lowest).
__device__ __forceinline__ unsigned gridHash(int gx, int gy, int gz,
                                             const SimParams &P) {
  unsigned x = (unsigned)gx & (P.gridSize[0] - 1u);
  unsigned y = (unsigned)gy & (P.gridSize[1] - 1u);
  unsigned z = (unsigned)gz & (P.gridSize[2] - 1u);
  if (mortonOrder(P)) return mortonSpread(x) | (mortonSpread(y) << 1) | (mortonSpread(z) << 2);
  return __umul24(__umul24(z, P.gridSize[1]), P.gridSize[0]) +
         __umul24(y, P.gridSize[0]) + x;
}

// The velocity and position update of particles_kernel.cu:55-59:
// vel += gravity * dt (fused), vel *= globalDamping, pos += vel * dt (fused).
__device__ __forceinline__ void advanceOne(float3 &p, float3 &v, float dt, const SimParams &P) {
  v.x = fmaf(P.gravity[0], dt, v.x);
  v.y = fmaf(P.gravity[1], dt, v.y);
  v.z = fmaf(P.gravity[2], dt, v.z);
  v.x = __fmul_rn(v.x, P.globalDamping);
  v.y = __fmul_rn(v.y, P.globalDamping);
  v.z = __fmul_rn(v.z, P.globalDamping);
  p.x = fmaf(v.x, dt, p.x);
  p.y = fmaf(v.y, dt, p.y);
  p.z = fmaf(v.z, dt, p.z);
}

// particles_kernel.cu:39-75 (integrate_functor) on one particle; r is the
// clamp radius (particleRadius, or pos.w in the polydisperse mode).
__device__ __forceinline__ void integrateOne(float3 &p, float3 &v, float dt,
                                             float r, const SimParams &P) {
  advanceOne(p, v, dt, P);
  const float bd = P.boundaryDamping;
  if (p.x > 1.0f - r) { p.x = 1.0f - r; v.x = __fmul_rn(v.x, bd); }
  if (p.x < -1.0f + r) { p.x = -1.0f + r; v.x = __fmul_rn(v.x, bd); }
  if (p.y > 1.0f - r) { p.y = 1.0f - r; v.y = __fmul_rn(v.y, bd); }
  if (p.z > 1.0f - r) { p.z = 1.0f - r; v.z = __fmul_rn(v.z, bd); }
  if (p.z < -1.0f + r) { p.z = -1.0f + r; v.z = __fmul_rn(v.z, bd); }
  if (p.y < -1.0f + r) { p.y = -1.0f + r; v.y = __fmul_rn(v.y, bd); }
}

// integrateOne with the box [lo, hi] instead of the reference's [-1, 1]^3
// (the batched scenes each have their own box); same faces in the same order.
__device__ __forceinline__ void integrateOneBox(float3 &p, float3 &v, float dt, float r,
                                                const SimParams &P, const float *lo,
                                                const float *hi) {
  advanceOne(p, v, dt, P);
  const float bd = P.boundaryDamping;
  if (p.x > hi[0] - r) { p.x = hi[0] - r; v.x = __fmul_rn(v.x, bd); }
  if (p.x < lo[0] + r) { p.x = lo[0] + r; v.x = __fmul_rn(v.x, bd); }
  if (p.y > hi[1] - r) { p.y = hi[1] - r; v.y = __fmul_rn(v.y, bd); }
  if (p.z > hi[2] - r) { p.z = hi[2] - r; v.z = __fmul_rn(v.z, bd); }
  if (p.z < lo[2] + r) { p.z = lo[2] + r; v.z = __fmul_rn(v.z, bd); }
  if (p.y < lo[1] + r) { p.y = lo[1] + r; v.y = __fmul_rn(v.y, bd); }
}

// The force of particles_kernel.cu:185-218 (collideSpheres) once the
// distance test has passed: rel = pB - pA, dist = |rel|, cd = rA + rB.
// norm = rel / dist (as rel * (1 / dist)); tanVel = relVel - dot(relVel,
// norm) * norm; force = -spring (cd - dist) norm + damping relVel + shear
// tanVel + attraction rel.  The fusions are the ones nvcc forms from the
// reference's expressions: in `a * b + c * d` the left product is fused
// with the right one as addend; in `x + a * b` the product is fused.
__device__ __forceinline__ float3 contactTerm(float3 rel, float dist, float cd,
                                              float3 vA, float3 vB,
                                              float attraction,
                                              const SimParams &P) {
  const float inv = __fdiv_rn(1.0f, dist);
  const float3 nrm = make_float3(__fmul_rn(rel.x, inv), __fmul_rn(rel.y, inv),
                                 __fmul_rn(rel.z, inv));
  const float3 rv = make_float3(__fsub_rn(vB.x, vA.x), __fsub_rn(vB.y, vA.y),
                                __fsub_rn(vB.z, vA.z));
  const float dn = fmaf(rv.z, nrm.z, fmaf(rv.x, nrm.x, __fmul_rn(rv.y, nrm.y)));
  const float3 tv = make_float3(fmaf(-nrm.x, dn, rv.x), fmaf(-nrm.y, dn, rv.y),
                                fmaf(-nrm.z, dn, rv.z));
  const float s = __fmul_rn(-P.spring, __fsub_rn(cd, dist));
  float3 f = make_float3(fmaf(s, nrm.x, __fmul_rn(P.damping, rv.x)),
                         fmaf(s, nrm.y, __fmul_rn(P.damping, rv.y)),
                         fmaf(s, nrm.z, __fmul_rn(P.damping, rv.z)));
  f.x = fmaf(tv.x, P.shear, f.x);
  f.y = fmaf(tv.y, P.shear, f.y);
  f.z = fmaf(tv.z, P.shear, f.z);
  f.x = fmaf(rel.x, attraction, f.x);
  f.y = fmaf(rel.y, attraction, f.y);
  f.z = fmaf(rel.z, attraction, f.z);
  return f;
}

// |rel|^2 as length() (cutil_math.cuh: sqrtf(dot(v, v))) evaluates it, the
// products fused into the sum as in contactTerm: sqrtf(pairDist2(rel)) is
// the pair distance.
__device__ __forceinline__ float pairDist2(float3 rel) {
  return fmaf(rel.z, rel.z, fmaf(rel.x, rel.x, __fmul_rn(rel.y, rel.y)));
}

__device__ __forceinline__ float pairDist(float3 rel) { return sqrtf(pairDist2(rel)); }

// A particle with a NaN or infinite coordinate takes part in no pair term:
// every squared distance to it is NaN or +inf, and neither passes the
// contact tests (`d2 < bound`, `dist < cd`, false for NaN and for +inf
// against a finite bound; an infinite bound needs an infinite radius and
// +inf < +inf is false too).  Its force is therefore +0.0, its partners get
// nothing from it, and skipping it leaves every sum unchanged.  Such
// particles arise in the reference's own arithmetic: two spheres of equal
// radius clamped into the same box corner coincide, dist = 0, and the
// normal rel / dist is NaN.
__device__ __forceinline__ bool inertPos(float3 p) {
  return !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z));
}
__device__ __forceinline__ bool inertPos(float4 p) {
  return !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z));
}

// Squared-distance bound for the contact test: d2 >= rejectBound(cd) implies
// sqrtf(d2) >= cd, so such a pair cannot pass `dist < cd` and is skipped
// without the (multi-instruction) IEEE square root.  Proof: the computed
// bound is >= cd^2 (1 - 2^-24)^2 (1 + 2.4e-6) > cd^2 (1 + 2.2e-6), hence
// sqrt(d2) > cd (1 + 1.1e-6) and the correctly rounded sqrtf(d2) > cd.
// Pairs below the bound take the exact test, so results are unchanged.
__device__ __forceinline__ float rejectBound(float cd) {
  return (cd * cd) * 1.0000025f;
}

// tileCnt[tile] += 1 for every calling lane, one atomic per distinct tile in
// the warp (consecutive sorted particles share tiles, so the atomics would
// otherwise queue on a few addresses).  Call from converged code or with the
// lanes that count.
__device__ __forceinline__ void countTile(unsigned *tileCnt, unsigned tile) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, tile);
  const unsigned lane = threadIdx.x & 31u;
  if ((peers & ((1u << lane) - 1u)) == 0u) atomicAdd(tileCnt + tile, (unsigned)__popc(peers));
}

}  // namespace fcdem
