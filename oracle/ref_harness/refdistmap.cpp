/*
 * refdistmap.cpp -- TEST INFRASTRUCTURE.  Builds the reference's own
 * distance-map query (cuda_addon/distancemap.cuh:118-302, the
 * DistanceMap<float,gpu> specialisation) and boundary response
 * (cuda_addon/boundaries.cuh:38-89) as host code, both included from the
 * reference tree at build time, with the reference's Vector3/AABB3 headers.
 * The DistanceMap primary template (inshape3dcore/grid/distancemap.h) pulls
 * in the unstructured grid and Eigen, so it is declared here instead; the
 * ParticleWorld<float, unified> the boundary functions read two parameters
 * from is a minimal stand-in with those two fields.  The integrate part of
 * d_integrateSystem (particledem_um.cu:604-631), which lives in a file that
 * needs the whole world set-up, is restated in fcref_um_integrate.
 */
#include "host_prelude.h"
#include <fcdefines.hpp>
#include <vector3.h>
#include <aabb3.h>

namespace i3d {
template <typename T, int memory = cpu> class DistanceMap;
template <typename T, int memory> struct ParticleWorld;
template <> struct ParticleWorld<float, unified> {
  struct Params { float particleRadius_; float boundaryDamping_; };
  Params *params_;
};
}  // namespace i3d

#define cudaCheckErrors(msg)
#include "distancemap.cuh"

#include "cutil_math.cuh"  // the float3 operators boundaries.cuh uses
using namespace i3d;
#include "boundaries.cuh"

namespace {
DistanceMap<float, gpu> makeMap(const float *distance, const float *cps, const float *coords,
                                const float *normals, const float vmin[3], const float vmax[3],
                                float cellSize, const int cells[3]) {
  DistanceMap<float, gpu> m;
  m.vertexCoords_ = (Vector3<float> *)coords;
  m.normals_ = (Vector3<float> *)normals;
  m.contactPoints_ = (Vector3<float> *)cps;
  m.distance_ = (float *)distance;
  m.stateFBM_ = nullptr;
  m.boundingBox_.vertices_[0] = Vector3<float>(vmin[0], vmin[1], vmin[2]);
  m.boundingBox_.vertices_[1] = Vector3<float>(vmax[0], vmax[1], vmax[2]);
  for (int k = 0; k < 3; ++k) m.cells_[k] = cells[k];
  m.cellSize_ = cellSize;
  return m;
}
}  // namespace

extern "C" {

/* queryMap for n points (3 floats each). */
void fcref_distmap_query(const float *distance, const float *cps, const float *coords,
                         const float vmin[3], const float vmax[3], float cellSize,
                         const int cells[3], const float *q, int n, float *dist, float *cp) {
  DistanceMap<float, gpu> m = makeMap(distance, cps, coords, nullptr, vmin, vmax, cellSize, cells);
  for (int i = 0; i < n; ++i) {
    vector3 query(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
    float d = 0.0f;
    vector3 c(0, 0, 0);
    m.queryMap(query, d, c);
    dist[i] = d;
    cp[3 * i] = c.x;
    cp[3 * i + 1] = c.y;
    cp[3 * i + 2] = c.z;
  }
}

/* d_integrateSystem of particledem_um.cu:604-638 on n particles (4 floats
 * each): the integrate restated, then the reference's d_checkBoundaryDistMap. */
void fcref_um_integrate(const float *distance, const float *cps, const float *coords,
                        const float *normals, const float vmin[3], const float vmax[3],
                        float cellSize, const int cells[3], float *pos, float *vel, int n,
                        const float gravity[3], float globalDamping, float dt, float radius,
                        float boundaryDamping) {
  DistanceMap<float, gpu> m =
      makeMap(distance, cps, coords, normals, vmin, vmax, cellSize, cells);
  ParticleWorld<float, unified>::Params prm{radius, boundaryDamping};
  ParticleWorld<float, unified> pw{&prm};
  for (int i = 0; i < n; ++i) {
    float3 p = make_float3(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
    float3 v = make_float3(vel[4 * i], vel[4 * i + 1], vel[4 * i + 2]);
    v.x = v.x + gravity[0] * dt; v.y = v.y + gravity[1] * dt; v.z = v.z + gravity[2] * dt;
    v.x = v.x * globalDamping; v.y = v.y * globalDamping; v.z = v.z * globalDamping;
    p.x = p.x + v.x * dt; p.y = p.y + v.y * dt; p.z = p.z + v.z * dt;
    d_checkBoundaryDistMap(p, v, &pw, &m);
    float w = pos[4 * i + 3];
    pos[4 * i] = p.x; pos[4 * i + 1] = p.y; pos[4 * i + 2] = p.z;
    vel[4 * i] = v.x; vel[4 * i + 1] = v.y; vel[4 * i + 2] = v.z; vel[4 * i + 3] = w;
  }
}

}  // extern "C"
