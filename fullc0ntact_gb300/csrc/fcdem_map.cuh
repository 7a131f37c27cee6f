// fcdem_map.cuh -- the device distance map (inshape3dcore/grid/distancemap.*,
// cuda_addon/distancemap.cuh:118-302) and the boundary response that reads it
// (cuda_addon/boundaries.cuh:38-63), shared by the distance-map kernels and
// the neural-SDF kernels.
//
// Map layout on the device: one float4 per lattice vertex, (distance, contact
// point x, y, z), vertex (i, j, k) at k*(cx+1)*(cy+1) + j*(cx+1) + i -- the
// reference keeps distance_ and contactPoints_ in separate arrays and the
// vertex coordinates in a third; here a corner is one 16-byte load and the
// coordinates are recomputed exactly as the host built them
// (vmin + i*cellSize in float, distancemap.cpp:214-226).
#pragma once
#include <cmath>
#include <cstdlib>

#include "fcdem_dem.cuh"

struct fcdemDistanceMap {
  float vmin[3], vmax[3];
  float cellSize;
  int cells[3];
  float4 *vert;  // device
  int device;
};

namespace fcdem {

struct MapView {
  float3 vmin, vmax;
  float cellSize;
  float invCell;  // (float)(1.0 / cellSize), as distancemap.cuh:173-174
  int cells[3];
  const float4 *__restrict__ vert;
};

inline MapView view(const fcdemDistanceMap *m) {
  MapView v;
  v.vmin = make_float3(m->vmin[0], m->vmin[1], m->vmin[2]);
  v.vmax = make_float3(m->vmax[0], m->vmax[1], m->vmax[2]);
  v.cellSize = m->cellSize;
  v.invCell = (float)(1.0 / (double)m->cellSize);
  for (int k = 0; k < 3; ++k) v.cells[k] = m->cells[k];
  v.vert = m->vert;
  return v;
}

// vmin + i * cellSize with two roundings, as the host lattice (no fused
// multiply-add: the reference computed it on the CPU).
__device__ __forceinline__ float vcoord(float vmin, int i, float cs) {
  return __fadd_rn(vmin, __fmul_rn((float)i, cs));
}

// DistanceMap<float,gpu>::queryMap (distancemap.cuh:154-191).  Returns the
// trilinear distance (5.0 outside the box) and contact point.  The cell index
// is clamped to cells-1 (the reference reads one vertex past the row for a
// query on the upper face).
__device__ __forceinline__ float queryMap(const MapView &M, float3 q, float3 &cp) {
  if (!(M.vmin.x <= q.x && q.x <= M.vmax.x && M.vmin.y <= q.y && q.y <= M.vmax.y &&
        M.vmin.z <= q.z && q.z <= M.vmax.z))
    return 5.0f;
  int x = (int)(fabsf(q.x - M.vmin.x) * M.invCell);
  int y = (int)(fabsf(q.y - M.vmin.y) * M.invCell);
  int z = (int)(fabsf(q.z - M.vmin.z) * M.invCell);
  x = min(max(x, 0), M.cells[0] - 1);
  y = min(max(y, 0), M.cells[1] - 1);
  z = min(max(z, 0), M.cells[2] - 1);
  // vertexIndices (distancemap.cuh:281-302)
  const int ix = M.cells[0] + 1;
  const int islice = (M.cells[0] + 1) * (M.cells[1] + 1);
  const int b = z * islice + y * ix + x;
  const float4 c0 = __ldg(M.vert + b), c1 = __ldg(M.vert + b + 1);
  const float4 c2 = __ldg(M.vert + b + ix + 1), c3 = __ldg(M.vert + b + ix);
  const float4 c4 = __ldg(M.vert + b + islice), c5 = __ldg(M.vert + b + islice + 1);
  const float4 c6 = __ldg(M.vert + b + ix + islice + 1), c7 = __ldg(M.vert + b + ix + islice);
  const float x0 = vcoord(M.vmin.x, x, M.cellSize), x1 = vcoord(M.vmin.x, x + 1, M.cellSize);
  const float y0 = vcoord(M.vmin.y, y, M.cellSize), y1 = vcoord(M.vmin.y, y + 1, M.cellSize);
  const float z0 = vcoord(M.vmin.z, z, M.cellSize), z1 = vcoord(M.vmin.z, z + 1, M.cellSize);
  const float xd = (q.x - x0) / (x1 - x0);
  const float yd = (q.y - y0) / (y1 - y0);
  const float zd = (q.z - z0) / (z1 - z0);
  // trilinearInterpolateDistance (distancemap.cuh:227-252).  In
  // `d0 * (1.0 - x_d) + d1 * x_d` the first product is double (1.0 is a
  // double literal), the second float * float; the sum is double, rounded to
  // float on assignment.  __fmul_rn keeps the float product unfused.
  const double wx = 1.0 - (double)xd, wy = 1.0 - (double)yd, wz = 1.0 - (double)zd;
  const float d00 = (float)((double)c0.x * wx + (double)__fmul_rn(c1.x, xd));
  const float d10 = (float)((double)c3.x * wx + (double)__fmul_rn(c2.x, xd));
  const float d01 = (float)((double)c4.x * wx + (double)__fmul_rn(c5.x, xd));
  const float d11 = (float)((double)c7.x * wx + (double)__fmul_rn(c6.x, xd));
  const float d0 = (float)((double)d00 * wy + (double)__fmul_rn(d10, yd));
  const float d1 = (float)((double)d01 * wy + (double)__fmul_rn(d11, yd));
  const float dist = (float)((double)d0 * wz + (double)__fmul_rn(d1, zd));
  // trilinearInterpolateCP (distancemap.cuh:254-279): Vector3<float> times the
  // weight converted to float.  Every sum a * w0 + b * w1 is written as
  // fmaf(a, w0, b * w1) with the second product rounded (lerp): each kernel
  // that inlines this function gets the same bits.
  const float fwx = (float)wx, fwy = (float)wy, fwz = (float)wz;
  auto lerp = [](float a, float w0, float b, float w1) {
    return fmaf(a, w0, __fmul_rn(b, w1));
  };
  float3 a00 = make_float3(lerp(c0.y, fwx, c1.y, xd), lerp(c0.z, fwx, c1.z, xd),
                           lerp(c0.w, fwx, c1.w, xd));
  float3 a10 = make_float3(lerp(c3.y, fwx, c2.y, xd), lerp(c3.z, fwx, c2.z, xd),
                           lerp(c3.w, fwx, c2.w, xd));
  float3 a01 = make_float3(lerp(c4.y, fwx, c5.y, xd), lerp(c4.z, fwx, c5.z, xd),
                           lerp(c4.w, fwx, c5.w, xd));
  float3 a11 = make_float3(lerp(c7.y, fwx, c6.y, xd), lerp(c7.z, fwx, c6.z, xd),
                           lerp(c7.w, fwx, c6.w, xd));
  float3 a0 = make_float3(lerp(a00.x, fwy, a10.x, yd), lerp(a00.y, fwy, a10.y, yd),
                          lerp(a00.z, fwy, a10.z, yd));
  float3 a1 = make_float3(lerp(a01.x, fwy, a11.x, yd), lerp(a01.y, fwy, a11.y, yd),
                          lerp(a01.z, fwy, a11.z, yd));
  cp = make_float3(lerp(a0.x, fwz, a1.x, zd), lerp(a0.y, fwz, a1.y, zd),
                   lerp(a0.z, fwz, a1.z, zd));
  return dist;
}

// checkDistMap (boundaries.cuh:38-63)
__device__ __forceinline__ void checkDistMap(const MapView &M, float radius, float bd,
                                             float3 &pos, float3 &vel) {
  float3 cp = make_float3(0.0f, 0.0f, 0.0f);
  const float dist = queryMap(M, pos, cp);
  if (dist < radius) {
    // the roundings are spelled out (fmaf, __fmul_rn) so that every kernel
    // inlining this function computes the same bits
    float3 n0 = make_float3(pos.x - cp.x, pos.y - cp.y, pos.z - cp.z);
    float invLen = rsqrtf(fmaf(n0.x, n0.x, fmaf(n0.y, n0.y, __fmul_rn(n0.z, n0.z))));
    float3 n = make_float3(__fmul_rn(n0.x, invLen), __fmul_rn(n0.y, invLen),
                           __fmul_rn(n0.z, invLen));
    float pen = radius - dist;
    float extra = (float)(0.1 * (double)radius);
    pos = make_float3(fmaf(n.x, pen, pos.x), fmaf(n.y, pen, pos.y), fmaf(n.z, pen, pos.z));
    pos = make_float3(fmaf(n.x, extra, pos.x), fmaf(n.y, extra, pos.y), fmaf(n.z, extra, pos.z));
    vel.x = __fmul_rn(vel.x, 0.5f * bd);
    vel.y = __fmul_rn(vel.y, 0.5f * bd);
    vel.z = __fmul_rn(vel.z, 0.7f * bd);
  }
}

// The velocity and position update of d_integrateSystem
// (particledem_um.cu:604-638).
__device__ __forceinline__ void umAdvance(float3 &p, float3 &v, float dt, const SimParams &P) {
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

// The rest of it: the map contact (when `mapTest`), the r = 1 cylinder
// around z, tested with the position before the map push, and the z planes
// at -1 and 10 (d_checkBoundaryDistMap, boundaries.cuh:65-89).  Roundings
// spelled out as in checkDistMap.
__device__ __forceinline__ void umBoundary(const MapView &M, bool mapTest, float r, float bd,
                                           float3 &p, float3 &v) {
  const float px0 = p.x, py0 = p.y;
  const float l2 = fmaf(px0, px0, __fmul_rn(py0, py0));  // + 0.0f * 0.0f: exact
  const float len = sqrtf(l2);
  if (mapTest) checkDistMap(M, r, bd, p, v);
  if (len > 1.0f) {
    const float pen = len - 1.0f;
    const float invLen = rsqrtf(l2);
    const float3 nn = make_float3(__fmul_rn(px0, invLen), __fmul_rn(py0, invLen), 0.0f);
    const float s = pen + r;
    p = make_float3(fmaf(-nn.x, s, p.x), fmaf(-nn.y, s, p.y), fmaf(-nn.z, s, p.z));
    v.x = __fmul_rn(v.x, bd);
    v.y = __fmul_rn(v.y, bd);
  }
  if (p.z > 10.0f - r) { p.z = 10.0f - r; v.z = __fmul_rn(v.z, bd); }
  if (p.z < -1.0f + r) { p.z = -1.0f + r; v.z = __fmul_rn(v.z, bd); }
}

// Inside the map box (where queryMap reads the map rather than 5.0).
__device__ __forceinline__ bool inMapBox(const MapView &M, float3 q) {
  return M.vmin.x <= q.x && q.x <= M.vmax.x && M.vmin.y <= q.y && q.y <= M.vmax.y &&
         M.vmin.z <= q.z && q.z <= M.vmax.z;
}

}  // namespace fcdem
