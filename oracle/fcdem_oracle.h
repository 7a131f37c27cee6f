/*
 * fcdem_oracle.h -- CPU restatement of FullC0ntact's particle-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  The tests compare the GPU implementation
 * against this library: only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark load it.  The product library never links or calls it.
 *
 * Every function restates one routine of the reference in plain C with the
 * same operation order, compiled with -ffp-contract=off so that results are
 * identical on x86-64 and aarch64.  Citations are file:line in the reference
 * tree (cuda_addon/..., inshape3dcore/...).
 */
#ifndef FCDEM_ORACLE_H
#define FCDEM_ORACLE_H

#include "../include/fcdem.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic of the restatement.  0 (default): every a*b+c with two
 * roundings, as the reference's code compiled for the host (the golden
 * fixtures) computes it.  1: the products that nvcc contracts in the
 * reference's CUDA build fused (fmaf), in the forms the GPU kernels of this
 * repository spell out -- integrate, the pair distance and the pair force.
 * Process-wide; the tests set it around a comparison. */
void orc_set_gpu_arithmetic(int on);

/* particles_kernel.cu:39-75 (integrate_functor).  radius_from_w selects the
 * polydisperse extension (clamp with pos.w instead of particleRadius). */
void orc_integrate(const SimParams *P, float *pos, float *vel, float dt,
                   unsigned n, int radius_from_w);

/* particles_kernel.cu:78-115 (calcGridPos, calcGridHash, calcHashD). */
void orc_calc_hash(const SimParams *P, unsigned *hash, unsigned *index,
                   const float *pos, unsigned n);

/* particleSystem.cu:265-270 (thrust::sort_by_key): stable ascending sort of
 * (key, value) pairs, restated as an LSD counting sort over 8-bit digits. */
void orc_sort_pairs(unsigned *keys, unsigned *vals, unsigned n);

/* particleSystem.cu:183-222 + particles_kernel.cu:119-182.  cellStart is set
 * to 0xffffffff first; cellEnd of empty cells is not touched. */
void orc_reorder(unsigned *cellStart, unsigned *cellEnd, float *sortedPos,
                 float *sortedVel, const unsigned *hash, const unsigned *index,
                 const float *oldPos, const float *oldVel, unsigned n,
                 unsigned numCells);

/* particles_kernel.cu:185-293 (collideSpheres, collideCell, collideD).
 * Writes newVel[index[i]] = (v + F, 0).  When force_out is not NULL it also
 * receives F (3 floats per particle, original order), the extra output of
 * particledem_um.cu:551,587.  with_collider = 0 drops the collider-sphere
 * term (particledem.cu / particledem_um.cu variants).  nthreads > 1 splits
 * the particles over POSIX threads; results do not depend on it. */
void orc_collide(const SimParams *P, float *newVel, float *force_out,
                 const float *sortedPos, const float *sortedVel,
                 const unsigned *index, const unsigned *cellStart,
                 const unsigned *cellEnd, unsigned n, int radius_from_w,
                 int with_collider, int nthreads);

/* Same as orc_collide, evaluated in double precision from the same float
 * inputs (same cells, same order).  newVel64 holds 4 doubles per particle. */
void orc_collide_f64(const SimParams *P, double *newVel64,
                     const float *sortedPos, const float *sortedVel,
                     const unsigned *index, const unsigned *cellStart,
                     const unsigned *cellEnd, unsigned n, int radius_from_w,
                     int with_collider, int nthreads);

/* One ParticleSystem::update (particleSystem.cpp:222-284): integrate, hash,
 * sort, reorder, collide.  Scratch arrays are caller-provided. */
void orc_update(const SimParams *P, float dt, float *pos, float *vel,
                float *sortedPos, float *sortedVel, unsigned *hash,
                unsigned *index, unsigned *cellStart, unsigned *cellEnd,
                unsigned n, int radius_from_w, int nthreads);

/* ---------------------------------------------------------------------- */
/* Distance map (inshape3dcore/grid/distancemap.{h,cpp},
 * cuda_addon/distancemap.cuh:118-302, cuda_addon/boundaries.cuh:38-89).
 * The vertex lattice is vmin + i*cellSize per axis (distancemap.cpp:214-226);
 * distance is float[V], contact points are 3 floats per vertex, vertex
 * (i,j,k) at k*(cx+1)*(cy+1) + j*(cx+1) + i. */
typedef struct orc_distmap {
  float vmin[3], vmax[3];
  float cellSize;
  int cells[3];
  const float *distance;
  const float *contactPoints;
} orc_distmap;

/* distancemap.cuh:154-191 (GPU variant: outside the box dist = 5.0).  The
 * cell index is clamped to cells-1 on each axis (the reference reads one
 * vertex past the row for a query exactly on the upper face). */
void orc_distmap_query(const orc_distmap *m, const float q[3], float *dist,
                       float cp[3]);

/* boundaries.cuh:38-63 (checkDistMap): push out of the mesh along
 * normalize(p - cp) and damp the velocity. */
void orc_check_distmap(const orc_distmap *m, float radius,
                       float boundaryDamping, float pos[3], float vel[3]);

/* particledem_um.cu:604-638 + boundaries.cuh:65-89: integrate with the
 * distance-map contact, the r = 1 cylinder and the z planes -1 and 10. */
void orc_integrate_distmap(const SimParams *P, const orc_distmap *m,
                           float *pos, float *vel, float dt, unsigned n,
                           int radius_from_w);

/* ---------------------------------------------------------------------- */
/* Batched scenes: one scene of a batch is one ParticleSystem with its own
 * parameters and its own box [lo, hi] instead of [-1, 1]^3.  The velocity
 * and position updates are fused multiply-adds, as nvcc builds the
 * reference's integrate (particles_kernel.cu:55-59, particledem_um.cu:625-630). */

/* particles_kernel.cu:39-75 with the faces of [lo, hi] in the reference's
 * order (+x, -x, +y, +z, -z, -y). */
void orc_integrate_box(const SimParams *P, const float lo[3], const float hi[3],
                       float *pos, float *vel, float dt, unsigned n,
                       int radius_from_w);

/* The integrate of a batched scene with an obstacle: the velocity and
 * position update of particledem_um.cu:604-638, checkDistMap
 * (boundaries.cuh:38-63) against the map m (NULL: no obstacle), then the
 * faces of [lo, hi].  *contacts (optional) receives the number of particles
 * the map pushed out. */
void orc_batch_obstacle_integrate(const SimParams *P, const float lo[3],
                                  const float hi[3], const orc_distmap *m,
                                  float *pos, float *vel, float dt, unsigned n,
                                  int radius_from_w, unsigned *contacts);

#ifdef __cplusplus
}
#endif

#endif
