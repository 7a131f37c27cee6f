// fcdem_distmap.cu -- distance-map boundary (inshape3dcore/grid/distancemap.*,
// cuda_addon/distancemap.cuh:118-302, cuda_addon/boundaries.cuh:38-89) and
// the particledem_um entry points that use it (cuda_addon/particledem_um.cu).
// The map types and the query live in fcdem_map.cuh.
#include <algorithm>
#include <cmath>
#include <vector>
#include <cstdlib>

#include "fcdem_map.cuh"

namespace fcdem {
namespace {

// d_integrateSystem + d_checkBoundaryDistMap (particledem_um.cu:604-638,
// boundaries.cuh:65-89): integrate, map contact, r = 1 cylinder around z,
// z planes at -1 and 10.  vel.w receives pos.w (particledem_um.cu:636).
// kCount: also the next step's calcHash and cell count (counting pipeline).
template <bool kCount>
__global__ void __launch_bounds__(256)
kIntegrateDistMap(float4 *__restrict__ pos, float4 *__restrict__ vel, float dt, unsigned n,
                  KParams kp, MapView M, int useMap, UmCount count) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SimParams &P = kp.p;
  float4 p4 = pos[i], v4 = vel[i];
  float3 p = make_float3(p4.x, p4.y, p4.z), v = make_float3(v4.x, v4.y, v4.z);
  const float r = kp.radiusFromW ? p4.w : P.particleRadius;
  umAdvance(p, v, dt, P);
  umBoundary(M, useMap != 0, r, P.boundaryDamping, p, v);
  pos[i] = make_float4(p.x, p.y, p.z, p4.w);
  vel[i] = make_float4(v.x, v.y, v.z, p4.w);
  if (kCount) {
    const int3 gp = gridPos(p.x, p.y, p.z, P);
    const unsigned h = gridHash(gp.x, gp.y, gp.z, P);
    count.hash[i] = h;
    count.rank[i] = atomicAdd(count.cnt + h, 1u);
    countTile(count.tileCnt, h >> 12);
  }
}

__global__ void __launch_bounds__(256)
kHashCount(const float4 *__restrict__ pos, unsigned n, KParams kp, UmCount count) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p4 = __ldg(pos + i);
  const int3 gp = gridPos(p4.x, p4.y, p4.z, kp.p);
  const unsigned h = gridHash(gp.x, gp.y, gp.z, kp.p);
  count.hash[i] = h;
  count.rank[i] = atomicAdd(count.cnt + h, 1u);
  countTile(count.tileCnt, h >> 12);
}

__global__ void __launch_bounds__(256)
kQueryMap(MapView M, const float4 *__restrict__ q, unsigned n, float *__restrict__ dist,
          float4 *__restrict__ cp) {
  unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = __ldg(q + i);
  float3 c = make_float3(0.0f, 0.0f, 0.0f);
  dist[i] = queryMap(M, make_float3(p.x, p.y, p.z), c);
  if (cp) cp[i] = make_float4(c.x, c.y, c.z, 0.0f);
}

// Exact signed distance and closest point of a torus around the z axis
// (major radius R, tube radius r) at every lattice vertex.
__global__ void __launch_bounds__(256)
kTorusMap(float4 *__restrict__ vert, int vx, int vy, int vz, float3 vmin, float cs, float R,
          float r) {
  const long long total = (long long)vx * vy * vz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % vx), j = (int)((t / vx) % vy), k = (int)(t / ((long long)vx * vy));
    const double px = (double)vcoord(vmin.x, i, cs), py = (double)vcoord(vmin.y, j, cs),
                 pz = (double)vcoord(vmin.z, k, cs);
    const double rho = sqrt(px * px + py * py);
    // closest point of the ring circle (any point of it for the axis)
    const double qx = rho > 0.0 ? R * px / rho : (double)R, qy = rho > 0.0 ? R * py / rho : 0.0;
    const double dx = px - qx, dy = py - qy, dz = pz;
    const double dq = sqrt(dx * dx + dy * dy + dz * dz);
    double cx, cy, cz;
    if (dq > 0.0) {
      cx = qx + r * dx / dq;
      cy = qy + r * dy / dq;
      cz = r * dz / dq;
    } else {  // on the ring circle: any point of the tube
      cx = qx * (1.0 + r / R);
      cy = qy * (1.0 + r / R);
      cz = 0.0;
    }
    vert[t] = make_float4((float)(dq - r), (float)cx, (float)cy, (float)cz);
  }
}

// Exact signed distance and closest point of a box with half-extents h whose
// edges and corners are rounded with radius rr (the box of half-extents
// h - rr grown by rr), centred at the origin, at every lattice vertex.
__global__ void __launch_bounds__(256)
kRoundedBoxMap(float4 *__restrict__ vert, int vx, int vy, int vz, float3 vmin, float cs,
               float3 h, float rr) {
  const long long total = (long long)vx * vy * vz;
  const double in[3] = {(double)h.x - rr, (double)h.y - rr, (double)h.z - rr};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % vx), j = (int)((t / vx) % vy), k = (int)(t / ((long long)vx * vy));
    const double p[3] = {(double)vcoord(vmin.x, i, cs), (double)vcoord(vmin.y, j, cs),
                         (double)vcoord(vmin.z, k, cs)};
    double c[3], q[3], o2 = 0.0, qmax = -1e300;
    int kmax = 0;
    for (int a = 0; a < 3; ++a) {
      c[a] = fmin(fmax(p[a], -in[a]), in[a]);  // closest point of the inner box
      q[a] = fabs(p[a]) - in[a];
      o2 += (p[a] - c[a]) * (p[a] - c[a]);
      if (q[a] > qmax) {
        qmax = q[a];
        kmax = a;
      }
    }
    double d, cp[3];
    if (o2 > 0.0) {  // outside the inner box: towards its closest point
      const double o = sqrt(o2);
      d = o - rr;
      for (int a = 0; a < 3; ++a) cp[a] = c[a] + rr * (p[a] - c[a]) / o;
    } else {  // inside it: the nearest flat face
      d = qmax - rr;
      for (int a = 0; a < 3; ++a) cp[a] = p[a];
      cp[kmax] = (p[kmax] < 0.0 ? -1.0 : 1.0) * (in[kmax] + rr);
    }
    vert[t] = make_float4((float)d, (float)cp[0], (float)cp[1], (float)cp[2]);
  }
}

// Closest point of triangle (a, b, c) to p: the region-based method of
// Ericson, Real-Time Collision Detection, section 5.1.5 (vertex, edge or face
// region from the barycentric signs).
__device__ __forceinline__ float3 closestOnTriangle(float3 p, float3 a, float3 b, float3 c) {
  const float3 ab = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
  const float3 ac = make_float3(c.x - a.x, c.y - a.y, c.z - a.z);
  const float3 ap = make_float3(p.x - a.x, p.y - a.y, p.z - a.z);
  auto dot = [](float3 u, float3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; };
  auto lerp = [](float3 o, float3 d, float t) {
    return make_float3(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z);
  };
  const float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.0f && d2 <= 0.0f) return a;
  const float3 bp = make_float3(p.x - b.x, p.y - b.y, p.z - b.z);
  const float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0f && d4 <= d3) return b;
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return lerp(a, ab, d1 / (d1 - d3));
  const float3 cp = make_float3(p.x - c.x, p.y - c.y, p.z - c.z);
  const float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0f && d5 <= d6) return c;
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return lerp(a, ac, d2 / (d2 - d6));
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
    const float3 bc = make_float3(c.x - b.x, c.y - b.y, c.z - b.z);
    return lerp(b, bc, (d4 - d3) / ((d4 - d3) + (d5 - d6)));
  }
  const float den = 1.0f / (va + vb + vc);
  const float v = vb * den, w = vc * den;
  return make_float3(a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w,
                     a.z + ab.z * v + ac.z * w);
}

// Solid angle of triangle (a, b, c) seen from p, signed by the triangle's
// orientation (Van Oosterom and Strackee, IEEE Trans. Biomed. Eng. 30, 1983).
__device__ __forceinline__ float solidAngle(float3 p, float3 a, float3 b, float3 c) {
  const float3 A = make_float3(a.x - p.x, a.y - p.y, a.z - p.z);
  const float3 B = make_float3(b.x - p.x, b.y - p.y, b.z - p.z);
  const float3 C = make_float3(c.x - p.x, c.y - p.y, c.z - p.z);
  const float la = sqrtf(A.x * A.x + A.y * A.y + A.z * A.z);
  const float lb = sqrtf(B.x * B.x + B.y * B.y + B.z * B.z);
  const float lc = sqrtf(C.x * C.x + C.y * C.y + C.z * C.z);
  const float det = A.x * (B.y * C.z - B.z * C.y) - A.y * (B.x * C.z - B.z * C.x) +
                    A.z * (B.x * C.y - B.y * C.x);
  const float den = la * lb * lc + (A.x * B.x + A.y * B.y + A.z * B.z) * lc +
                    (A.x * C.x + A.y * C.y + A.z * C.z) * lb +
                    (B.x * C.x + B.y * C.y + B.z * C.z) * la;
  return 2.0f * atan2f(det, den);
}

constexpr int kMeshChunk = 256;

// Distance map of a closed, outward-oriented triangle mesh: at every lattice
// vertex the distance to the closest point of the mesh, negative inside (the
// generalized winding number, the summed solid angles over 4 pi, above 1/2),
// and that closest point as the contact point -- what DistanceMapMesh::
// ComputeDistance (distancegridcgal.hpp:36-69) stores.  One thread per
// vertex; the triangles go through shared memory in chunks.
__global__ void __launch_bounds__(128)
kMeshMap(float4 *__restrict__ vert, int vx, int vy, int vz, float3 vmin, float cs,
         const float4 *__restrict__ tri, unsigned nt) {
  __shared__ float4 sTri[kMeshChunk * 3];
  const long long total = (long long)vx * vy * vz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = t < total;
  float3 p = make_float3(0.0f, 0.0f, 0.0f);
  if (valid) {
    const int i = (int)(t % vx), j = (int)((t / vx) % vy), k = (int)(t / ((long long)vx * vy));
    p = make_float3(vcoord(vmin.x, i, cs), vcoord(vmin.y, j, cs), vcoord(vmin.z, k, cs));
  }
  float best = 3.4e38f;
  float3 bestCp = p;
  float omega = 0.0f;
  for (unsigned base = 0; base < nt; base += kMeshChunk) {
    const unsigned cnt = min((unsigned)kMeshChunk, nt - base);
    __syncthreads();
    for (unsigned e = threadIdx.x; e < cnt * 3; e += blockDim.x) sTri[e] = __ldg(tri + base * 3 + e);
    __syncthreads();
    if (!valid) continue;
    for (unsigned q = 0; q < cnt; ++q) {
      const float4 a4 = sTri[3 * q], b4 = sTri[3 * q + 1], c4 = sTri[3 * q + 2];
      const float3 a = make_float3(a4.x, a4.y, a4.z), b = make_float3(b4.x, b4.y, b4.z),
                   c = make_float3(c4.x, c4.y, c4.z);
      const float3 cp = closestOnTriangle(p, a, b, c);
      const float dx = p.x - cp.x, dy = p.y - cp.y, dz = p.z - cp.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < best) {
        best = d2;
        bestCp = cp;
      }
      omega += solidAngle(p, a, b, c);
    }
  }
  if (!valid) return;
  const bool inside = omega > 2.0f * 3.14159265358979f;  // winding number > 1/2
  const float d = sqrtf(best);
  vert[t] = make_float4(inside ? -d : d, bestCp.x, bestCp.y, bestCp.z);
}

// d_integrateRigidBody (particledem_um.cu:640-718), one thread per body:
// the body's velocity takes gravity and the global damping, its centre moves
// by v dt; of both, only z is stored (the reference writes vel_.z and com_.z
// and nothing else), and the body's member particles are translated by the
// full v dt with w = 1.  The reference's box clamp acts on its local copies
// after the stores and changes nothing; it is left out.  The reference moves
// particles 0..2 for body 0 and 3..5 for every other body; here each body
// moves the members listed in its own indices[0 .. numParticles).
__global__ void __launch_bounds__(128)
kIntegrateRigidBodies(fcdemRigidBody *__restrict__ bodies, unsigned nb,
                      float4 *__restrict__ pos, unsigned np, float dt, KParams kp) {
  const unsigned b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const SimParams &P = kp.p;
  fcdemRigidBody rb = bodies[b];
  float3 v = make_float3(rb.vel[0], rb.vel[1], rb.vel[2]);
  v.x = fmaf(P.gravity[0], dt, v.x);
  v.y = fmaf(P.gravity[1], dt, v.y);
  v.z = fmaf(P.gravity[2], dt, v.z);
  v.x = __fmul_rn(v.x, P.globalDamping);
  v.y = __fmul_rn(v.y, P.globalDamping);
  v.z = __fmul_rn(v.z, P.globalDamping);
  bodies[b].vel[2] = v.z;
  bodies[b].com[2] = fmaf(v.z, dt, rb.com[2]);
  const int m = rb.numParticles < 3 ? rb.numParticles : 3;
  for (int k = 0; k < m; ++k) {
    const int q = rb.indices[k];
    if (q < 0 || (unsigned)q >= np) continue;
    const float4 p = pos[q];
    pos[q] = make_float4(fmaf(v.x, dt, p.x), fmaf(v.y, dt, p.y), fmaf(v.z, dt, p.z), 1.0f);
  }
}

}  // namespace
}  // namespace fcdem

namespace fcdem {

bool umHashCount(const float4 *pos, unsigned n, const KParams &kp, const UmCount &count) {
  kHashCount<<<(n + 255) / 256, 256, 0, curStream()>>>(pos, n, kp, count);
  return launchOk();
}

bool mapIntegrate(float4 *pos, float4 *vel, float dt, unsigned n, const KParams &kp,
                  const fcdemDistanceMap *map, const UmCount *count) {
  MapView M{};
  if (map) M = view(map);
  const unsigned blocks = (n + 255) / 256;
  if (count)
    kIntegrateDistMap<true><<<blocks, 256, 0, curStream()>>>(pos, vel, dt, n, kp, M,
                                                             map ? 1 : 0, *count);
  else
    kIntegrateDistMap<false><<<blocks, 256, 0, curStream()>>>(pos, vel, dt, n, kp, M,
                                                              map ? 1 : 0, UmCount{});
  return launchOk();
}

}  // namespace fcdem

using namespace fcdem;

extern "C" {

fcdemDistanceMap *fcdemDistMapCreate(const float *distance, const float *contactPoints,
                                     const float vmin[3], const float vmax[3],
                                     float cellSize, const int cells[3]) {
  if (!vmin || !vmax || !cells || cells[0] < 1 || cells[1] < 1 || cells[2] < 1 ||
      !(cellSize > 0.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return nullptr;
  }
  fcdemDistanceMap *m = new fcdemDistanceMap();
  for (int k = 0; k < 3; ++k) {
    m->vmin[k] = vmin[k];
    m->vmax[k] = vmax[k];
    m->cells[k] = cells[k];
  }
  m->cellSize = cellSize;
  cudaGetDevice(&m->device);
  const size_t nv = (size_t)(cells[0] + 1) * (cells[1] + 1) * (cells[2] + 1);
  if (cudaMalloc(&m->vert, nv * sizeof(float4)) != cudaSuccess) {
    cudaGetLastError();
    delete m;
    setError(FCDEM_ERR_ALLOC);
    return nullptr;
  }
  if (distance && contactPoints) {  // host arrays in the reference's layout
    float4 *h = (float4 *)std::malloc(nv * sizeof(float4));
    if (!h) {
      cudaFree(m->vert);
      delete m;
      setError(FCDEM_ERR_ALLOC);
      return nullptr;
    }
    for (size_t v = 0; v < nv; ++v)
      h[v] = make_float4(distance[v], contactPoints[3 * v], contactPoints[3 * v + 1],
                         contactPoints[3 * v + 2]);
    cudaOk(cudaMemcpy(m->vert, h, nv * sizeof(float4), cudaMemcpyHostToDevice));
    std::free(h);
  } else {
    cudaOk(cudaMemset(m->vert, 0, nv * sizeof(float4)));
  }
  return m;
}

fcdemDistanceMap *fcdemDistMapTorus(float majorRadius, float tubeRadius, int cellsPerAxis,
                                    float margin) {
  if (!(majorRadius > tubeRadius) || !(tubeRadius > 0.0f) || cellsPerAxis < 1) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return nullptr;
  }
  // Cubic cells over the torus box plus the margin: x, y span
  // +-(R + r + margin); z spans +-(r + margin) rounded up to whole cells.
  const float ex = majorRadius + tubeRadius + margin;
  const float cs = 2.0f * ex / (float)cellsPerAxis;
  int cz = (int)std::ceil(2.0f * (tubeRadius + margin) / cs);
  if (cz < 1) cz = 1;
  const float vmin[3] = {-ex, -ex, -0.5f * cz * cs};
  const float vmax[3] = {vmin[0] + cellsPerAxis * cs, vmin[1] + cellsPerAxis * cs,
                         vmin[2] + cz * cs};
  const int cells[3] = {cellsPerAxis, cellsPerAxis, cz};
  fcdemDistanceMap *m = fcdemDistMapCreate(nullptr, nullptr, vmin, vmax, cs, cells);
  if (!m) return nullptr;
  kTorusMap<<<numSms() * 8, 256, 0, curStream()>>>(m->vert, cells[0] + 1, cells[1] + 1,
                                              cells[2] + 1,
                                              make_float3(vmin[0], vmin[1], vmin[2]), cs,
                                              majorRadius, tubeRadius);
  launchOk();
  return m;
}

fcdemDistanceMap *fcdemDistMapRoundedBox(const float halfExtents[3], float rounding,
                                         int cellsPerAxis, float margin) {
  if (!halfExtents || cellsPerAxis < 1 || !(rounding >= 0.0f) || !(margin >= 0.0f) ||
      !(halfExtents[0] > rounding) || !(halfExtents[1] > rounding) ||
      !(halfExtents[2] > rounding)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return nullptr;
  }
  // cubic cells: the largest axis gets cellsPerAxis cells over
  // +-(h + margin), the others whole cells covering theirs
  float ex[3], big = 0.0f;
  for (int a = 0; a < 3; ++a) {
    ex[a] = halfExtents[a] + margin;
    big = std::fmax(big, ex[a]);
  }
  const float cs = 2.0f * big / (float)cellsPerAxis;
  int cells[3];
  float vmin[3], vmax[3];
  for (int a = 0; a < 3; ++a) {
    cells[a] = (int)std::ceil(2.0f * ex[a] / cs);
    if (cells[a] < 1) cells[a] = 1;
    vmin[a] = -0.5f * cells[a] * cs;
    vmax[a] = vmin[a] + cells[a] * cs;
  }
  fcdemDistanceMap *m = fcdemDistMapCreate(nullptr, nullptr, vmin, vmax, cs, cells);
  if (!m) return nullptr;
  kRoundedBoxMap<<<numSms() * 8, 256, 0, curStream()>>>(
      m->vert, cells[0] + 1, cells[1] + 1, cells[2] + 1,
      make_float3(vmin[0], vmin[1], vmin[2]), cs,
      make_float3(halfExtents[0], halfExtents[1], halfExtents[2]), rounding);
  launchOk();
  return m;
}

fcdemDistanceMap *fcdemDistMapFromMesh(const float *vertices3, uint numVertices,
                                       const uint *triangles3, uint numTriangles,
                                       int cellsPerAxis, float margin) {
  if (!vertices3 || !triangles3 || numVertices < 3 || numTriangles < 1 || cellsPerAxis < 1 ||
      !(margin >= 0.0f)) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return nullptr;
  }
  float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint v = 0; v < numVertices; ++v)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::fmin(lo[a], vertices3[3 * v + a]);
      hi[a] = std::fmax(hi[a], vertices3[3 * v + a]);
    }
  std::vector<float4> tri((size_t)numTriangles * 3);
  for (uint t = 0; t < numTriangles; ++t)
    for (int c = 0; c < 3; ++c) {
      const uint v = triangles3[3 * t + c];
      if (v >= numVertices) { setError(FCDEM_ERR_INVALID_VALUE); return nullptr; }
      tri[3 * t + c] = make_float4(vertices3[3 * v], vertices3[3 * v + 1], vertices3[3 * v + 2], 0.0f);
    }
  // cubic cells over the mesh box plus the margin, centred on the box: the
  // largest axis cut into cellsPerAxis cells, the others into whole cells
  float centre[3], ex[3], big = 0.0f;
  for (int a = 0; a < 3; ++a) {
    centre[a] = 0.5f * (lo[a] + hi[a]);
    ex[a] = 0.5f * (hi[a] - lo[a]) + margin;
    big = std::fmax(big, ex[a]);
  }
  if (!(big > 0.0f)) { setError(FCDEM_ERR_INVALID_VALUE); return nullptr; }
  const float cs = 2.0f * big / (float)cellsPerAxis;
  int cells[3];
  float vmin[3], vmax[3];
  for (int a = 0; a < 3; ++a) {
    cells[a] = std::max(1, (int)std::ceil(2.0f * ex[a] / cs));
    vmin[a] = centre[a] - 0.5f * cells[a] * cs;
    vmax[a] = vmin[a] + cells[a] * cs;
  }
  fcdemDistanceMap *m = fcdemDistMapCreate(nullptr, nullptr, vmin, vmax, cs, cells);
  if (!m) return nullptr;
  float4 *dTri = nullptr;
  if (cudaMalloc(&dTri, tri.size() * sizeof(float4)) != cudaSuccess) {
    cudaGetLastError();
    fcdemDistMapDestroy(m);
    setError(FCDEM_ERR_ALLOC);
    return nullptr;
  }
  bool ok = cudaOk(cudaMemcpy(dTri, tri.data(), tri.size() * sizeof(float4), cudaMemcpyHostToDevice));
  const long long total = (long long)(cells[0] + 1) * (cells[1] + 1) * (cells[2] + 1);
  if (ok) {
    kMeshMap<<<(unsigned)((total + 127) / 128), 128, 0, curStream()>>>(
        m->vert, cells[0] + 1, cells[1] + 1, cells[2] + 1, make_float3(vmin[0], vmin[1], vmin[2]),
        cs, dTri, numTriangles);
    ok = launchOk() && cudaOk(cudaStreamSynchronize(curStream()));
  }
  cudaFree(dTri);
  if (!ok) {
    fcdemDistMapDestroy(m);
    return nullptr;
  }
  return m;
}

void fcdemDistMapDestroy(fcdemDistanceMap *m) {
  if (!m) return;
  cudaOk(cudaFree(m->vert));
  delete m;
}

void fcdemDistMapGeometry(const fcdemDistanceMap *m, float vmin[3], float vmax[3],
                          float *cellSize, int cells[3]) {
  if (!m) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  for (int k = 0; k < 3; ++k) {
    if (vmin) vmin[k] = m->vmin[k];
    if (vmax) vmax[k] = m->vmax[k];
    if (cells) cells[k] = m->cells[k];
  }
  if (cellSize) *cellSize = m->cellSize;
}

void fcdemDistMapVertices(const fcdemDistanceMap *m, float *vertices4) {
  if (!m || !vertices4) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  const size_t nv = (size_t)(m->cells[0] + 1) * (m->cells[1] + 1) * (m->cells[2] + 1);
  cudaOk(cudaMemcpy(vertices4, m->vert, nv * sizeof(float4), cudaMemcpyDeviceToHost));
}

void fcdemDistMapQuery(const fcdemDistanceMap *m, const float *queries4, unsigned n,
                       float *dist, float *cp4) {
  if (!m || (n && (!queries4 || !dist))) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  if (n == 0) return;
  kQueryMap<<<(n + 255) / 256, 256, 0, curStream()>>>(view(m), (const float4 *)queries4, n,
                                                      dist, (float4 *)cp4);
  launchOk();
}

void fcdemUM_integrateSystem(float *pos, float *vel, float deltaTime, uint numParticles,
                             const fcdemDistanceMap *map) {
  Context &c = ctx();
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return; }
  if (numParticles == 0) return;
  if (!pos || !vel) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  mapIntegrate((float4 *)pos, (float4 *)vel, deltaTime, numParticles, kparams(c), map, nullptr);
}

void fcdemUM_integrateRigidBodies(fcdemRigidBody *bodies, uint numBodies, float *pos,
                                  uint numParticles, float deltaTime) {
  Context &c = ctx();
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return; }
  if (numBodies == 0) return;
  if (!bodies || !pos) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  kIntegrateRigidBodies<<<(numBodies + 127) / 128, 128, 0, curStream()>>>(
      bodies, numBodies, (float4 *)pos, numParticles, deltaTime, kparams(c));
  launchOk();
}

void fcdemUM_evalForces(float *newVel, float *force, float *sortedPos, float *sortedVel,
                        uint *gridParticleIndex, uint *cellStart, uint *cellEnd,
                        uint numParticles, uint numCells) {
  Context &c = ctx();
  if (!c.haveParams) { setError(FCDEM_ERR_NO_PARAMS); return; }
  if (numParticles == 0) return;
  if (!newVel || !force || !sortedPos || !sortedVel || !gridParticleIndex || !cellStart ||
      !cellEnd) {
    setError(FCDEM_ERR_INVALID_VALUE);
    return;
  }
  unsigned long long cells =
      (unsigned long long)c.params.gridSize[0] * c.params.gridSize[1] * c.params.gridSize[2];
  if (cells > numCells) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  CellRanges cr;
  cr.start = cellStart;
  cr.end = cellEnd;
  CollideOut out;
  out.force = (float3 *)force;
  launchCollide(0, false, (float4 *)newVel, (const float4 *)sortedPos,
                (const float4 *)sortedVel, gridParticleIndex, cr, numParticles, kparams(c),
                out);
}

void fcdemUM_reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd, float *sortedPos,
                                         float *sortedVel, uint *gridParticleHash,
                                         uint *gridParticleIndex, float *oldPos, float *oldVel,
                                         uint numParticles, uint numCells) {
  // particledem_um.cu:442-454 resets cellEnd as well as cellStart
  if (!cellEnd) { setError(FCDEM_ERR_INVALID_VALUE); return; }
  fillU32(ctx(), cellEnd, numCells, 0xffffffffu);
  reorderDataAndFindCellStart(cellStart, cellEnd, sortedPos, sortedVel, gridParticleHash,
                              gridParticleIndex, oldPos, oldVel, numParticles, numCells);
}

}  // extern "C"
