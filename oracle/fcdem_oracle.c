/*
 * fcdem_oracle.c -- CPU restatement of FullC0ntact's particle-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU restatement the GPU kernels are tested
 * against.  Only tests/, the smoke check and the CPU-baseline leg of bench.py
 * load it.
 *
 * Build with -ffp-contract=off (see oracle/Makefile): every a*b+c below is
 * two roundings, on every host architecture.
 */
#include "fcdem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } f3;

/* Arithmetic mode (orc_set_gpu_arithmetic): 0 evaluates every a*b+c with
 * two roundings, as the reference's code built for the host does; 1 fuses
 * the products the reference's CUDA build contracts (nvcc's default), in
 * the forms the GPU kernels of this repository spell out with fmaf. */
static int g_gpu_arith = 0;

void orc_set_gpu_arithmetic(int on) { g_gpu_arith = on ? 1 : 0; }

static inline f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }

/* PTX cvt.rzi.s32.f32 semantics for the float->int conversion of the grid
 * position (particles_kernel.cu:81-83 assigns floor(...) to an int):
 * NaN -> 0, saturating at the int range. */
static inline int f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return 2147483647;
  if (f < -2147483648.0f) return (-2147483647 - 1);
  return (int)f;
}

/* __umul24: product of the low 24 bits of both operands, low 32 bits kept. */
static inline unsigned umul24(unsigned a, unsigned b) {
  return (a & 0xffffffu) * (b & 0xffffffu);
}

/* particles_kernel.cu:78-85 */
static inline void grid_pos(const SimParams *P, float px, float py, float pz,
                            int g[3]) {
  g[0] = f2i_sat(floorf((px - P->worldOrigin[0]) / P->cellSize[0]));
  g[1] = f2i_sat(floorf((py - P->worldOrigin[1]) / P->cellSize[1]));
  g[2] = f2i_sat(floorf((pz - P->worldOrigin[2]) / P->cellSize[2]));
}

/* particles_kernel.cu:88-94 */
static inline unsigned grid_hash(const SimParams *P, int gx, int gy, int gz) {
  unsigned x = (unsigned)gx & (P->gridSize[0] - 1u);
  unsigned y = (unsigned)gy & (P->gridSize[1] - 1u);
  unsigned z = (unsigned)gz & (P->gridSize[2] - 1u);
  return umul24(umul24(z, P->gridSize[1]), P->gridSize[0]) +
         umul24(y, P->gridSize[0]) + x;
}

/* ---------------------------------------------------------------------- */
void orc_integrate(const SimParams *P, float *pos, float *vel, float dt,
                   unsigned n, int radius_from_w) {
  for (unsigned i = 0; i < n; ++i) {
    float *p4 = pos + 4 * (size_t)i, *v4 = vel + 4 * (size_t)i;
    float px = p4[0], py = p4[1], pz = p4[2];
    float vx = v4[0], vy = v4[1], vz = v4[2];
    float r = radius_from_w ? p4[3] : P->particleRadius;
    float bd = P->boundaryDamping;
    /* vel += gravity * deltaTime; vel *= globalDamping; pos += vel * deltaTime
     * (particles_kernel.cu:55-59) */
    if (g_gpu_arith) {
      vx = fmaf(P->gravity[0], dt, vx);
      vy = fmaf(P->gravity[1], dt, vy);
      vz = fmaf(P->gravity[2], dt, vz);
    } else {
      vx = vx + P->gravity[0] * dt;
      vy = vy + P->gravity[1] * dt;
      vz = vz + P->gravity[2] * dt;
    }
    vx = vx * P->globalDamping;
    vy = vy * P->globalDamping;
    vz = vz * P->globalDamping;
    if (g_gpu_arith) {
      px = fmaf(vx, dt, px);
      py = fmaf(vy, dt, py);
      pz = fmaf(vz, dt, pz);
    } else {
      px = px + vx * dt;
      py = py + vy * dt;
      pz = pz + vz * dt;
    }
    /* faces in the reference's order: +x, -x, +y, +z, -z, -y */
    if (px > 1.0f - r) { px = 1.0f - r; vx = vx * bd; }
    if (px < -1.0f + r) { px = -1.0f + r; vx = vx * bd; }
    if (py > 1.0f - r) { py = 1.0f - r; vy = vy * bd; }
    if (pz > 1.0f - r) { pz = 1.0f - r; vz = vz * bd; }
    if (pz < -1.0f + r) { pz = -1.0f + r; vz = vz * bd; }
    if (py < -1.0f + r) { py = -1.0f + r; vy = vy * bd; }
    p4[0] = px; p4[1] = py; p4[2] = pz;          /* w kept */
    v4[0] = vx; v4[1] = vy; v4[2] = vz;          /* w kept */
  }
}

/* ---------------------------------------------------------------------- */
void orc_calc_hash(const SimParams *P, unsigned *hash, unsigned *index,
                   const float *pos, unsigned n) {
  for (unsigned i = 0; i < n; ++i) {
    int g[3];
    grid_pos(P, pos[4 * (size_t)i], pos[4 * (size_t)i + 1],
             pos[4 * (size_t)i + 2], g);
    hash[i] = grid_hash(P, g[0], g[1], g[2]);
    index[i] = i;
  }
}

/* ---------------------------------------------------------------------- */
void orc_sort_pairs(unsigned *keys, unsigned *vals, unsigned n) {
  if (n < 2) return;
  unsigned *k2 = (unsigned *)malloc(sizeof(unsigned) * (size_t)n);
  unsigned *v2 = (unsigned *)malloc(sizeof(unsigned) * (size_t)n);
  unsigned *ka = keys, *va = vals, *kb = k2, *vb = v2;
  for (int shift = 0; shift < 32; shift += 8) {
    size_t count[257];
    memset(count, 0, sizeof(count));
    for (unsigned i = 0; i < n; ++i) count[((ka[i] >> shift) & 255u) + 1]++;
    int trivial = 0;
    for (int d = 0; d < 256; ++d)
      if (count[d + 1] == n) trivial = 1;
    if (trivial) continue; /* one digit value: the pass is the identity */
    for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
    for (unsigned i = 0; i < n; ++i) { /* ascending i: stable */
      size_t dst = count[(ka[i] >> shift) & 255u]++;
      kb[dst] = ka[i];
      vb[dst] = va[i];
    }
    unsigned *t = ka; ka = kb; kb = t;
    t = va; va = vb; vb = t;
  }
  if (ka != keys) {
    memcpy(keys, ka, sizeof(unsigned) * (size_t)n);
    memcpy(vals, va, sizeof(unsigned) * (size_t)n);
  }
  free(k2);
  free(v2);
}

/* ---------------------------------------------------------------------- */
void orc_reorder(unsigned *cellStart, unsigned *cellEnd, float *sortedPos,
                 float *sortedVel, const unsigned *hash, const unsigned *index,
                 const float *oldPos, const float *oldVel, unsigned n,
                 unsigned numCells) {
  memset(cellStart, 0xff, sizeof(unsigned) * (size_t)numCells);
  for (unsigned i = 0; i < n; ++i) {
    unsigned h = hash[i];
    if (i == 0 || h != hash[i - 1]) {
      cellStart[h] = i;
      if (i > 0) cellEnd[hash[i - 1]] = i;
    }
    if (i == n - 1) cellEnd[h] = i + 1;
    unsigned s = index[i];
    memcpy(sortedPos + 4 * (size_t)i, oldPos + 4 * (size_t)s, 16);
    memcpy(sortedVel + 4 * (size_t)i, oldVel + 4 * (size_t)s, 16);
  }
}

/* ---------------------------------------------------------------------- */
/* particles_kernel.cu:185-218 with the products nvcc contracts fused: in
 * `a * b + c * d` the left product is fused with the right one as addend,
 * in `x + a * b` the product is fused (dot products, the tangential
 * velocity, the force sum). */
static inline f3 sphere_term_fused(f3 pA, f3 pB, f3 vA, f3 vB, float rA, float rB,
                                   float attraction, const SimParams *P) {
  f3 rel = mk3(pB.x - pA.x, pB.y - pA.y, pB.z - pA.z);
  float dist = sqrtf(fmaf(rel.z, rel.z, fmaf(rel.x, rel.x, rel.y * rel.y)));
  float cd = rA + rB;
  f3 f = mk3(0.0f, 0.0f, 0.0f);
  if (dist < cd) {
    float inv = 1.0f / dist;
    f3 nrm = mk3(rel.x * inv, rel.y * inv, rel.z * inv);
    f3 rv = mk3(vB.x - vA.x, vB.y - vA.y, vB.z - vA.z);
    float dn = fmaf(rv.z, nrm.z, fmaf(rv.x, nrm.x, rv.y * nrm.y));
    f3 tv = mk3(fmaf(-nrm.x, dn, rv.x), fmaf(-nrm.y, dn, rv.y), fmaf(-nrm.z, dn, rv.z));
    float s = -P->spring * (cd - dist);
    f.x = fmaf(s, nrm.x, P->damping * rv.x);
    f.y = fmaf(s, nrm.y, P->damping * rv.y);
    f.z = fmaf(s, nrm.z, P->damping * rv.z);
    f.x = fmaf(tv.x, P->shear, f.x);
    f.y = fmaf(tv.y, P->shear, f.y);
    f.z = fmaf(tv.z, P->shear, f.z);
    f.x = fmaf(rel.x, attraction, f.x);
    f.y = fmaf(rel.y, attraction, f.y);
    f.z = fmaf(rel.z, attraction, f.z);
  }
  return f;
}

/* particles_kernel.cu:185-218, float.  Returns the pair term. */
static inline f3 sphere_term(f3 pA, f3 pB, f3 vA, f3 vB, float rA, float rB,
                             float attraction, const SimParams *P) {
  if (g_gpu_arith) return sphere_term_fused(pA, pB, vA, vB, rA, rB, attraction, P);
  f3 rel = mk3(pB.x - pA.x, pB.y - pA.y, pB.z - pA.z);
  float dist = sqrtf(rel.x * rel.x + rel.y * rel.y + rel.z * rel.z);
  float cd = rA + rB;
  f3 f = mk3(0.0f, 0.0f, 0.0f);
  if (dist < cd) {
    float inv = 1.0f / dist;
    f3 nrm = mk3(rel.x * inv, rel.y * inv, rel.z * inv);
    f3 rv = mk3(vB.x - vA.x, vB.y - vA.y, vB.z - vA.z);
    float dn = rv.x * nrm.x + rv.y * nrm.y + rv.z * nrm.z;
    f3 tv = mk3(rv.x - nrm.x * dn, rv.y - nrm.y * dn, rv.z - nrm.z * dn);
    float s = -P->spring * (cd - dist);
    f.x = nrm.x * s; f.y = nrm.y * s; f.z = nrm.z * s;
    f.x = f.x + rv.x * P->damping;
    f.y = f.y + rv.y * P->damping;
    f.z = f.z + rv.z * P->damping;
    f.x = f.x + tv.x * P->shear;
    f.y = f.y + tv.y * P->shear;
    f.z = f.z + tv.z * P->shear;
    f.x = f.x + rel.x * attraction;
    f.y = f.y + rel.y * attraction;
    f.z = f.z + rel.z * attraction;
  }
  return f;
}

typedef struct {
  const SimParams *P;
  float *newVel;
  float *force_out;
  double *newVel64;
  const float *sp, *sv;
  const unsigned *index, *cs, *ce;
  unsigned n, begin, end;
  int radius_from_w, with_collider;
} collide_job;

static void collide_range(const collide_job *J) {
  const SimParams *P = J->P;
  for (unsigned i = J->begin; i < J->end; ++i) {
    const float *p4 = J->sp + 4 * (size_t)i, *v4 = J->sv + 4 * (size_t)i;
    f3 pos = mk3(p4[0], p4[1], p4[2]);
    f3 vel = mk3(v4[0], v4[1], v4[2]);
    float ri = J->radius_from_w ? p4[3] : P->particleRadius;
    int g[3];
    grid_pos(P, pos.x, pos.y, pos.z, g);
    f3 force = mk3(0.0f, 0.0f, 0.0f);
    for (int z = -1; z <= 1; ++z)
      for (int y = -1; y <= 1; ++y)
        for (int x = -1; x <= 1; ++x) {
          /* collideCell, particles_kernel.cu:223-253 */
          unsigned h = grid_hash(P, g[0] + x, g[1] + y, g[2] + z);
          unsigned s = J->cs[h];
          f3 cf = mk3(0.0f, 0.0f, 0.0f);
          if (s != 0xffffffffu) {
            unsigned e = J->ce[h];
            for (unsigned j = s; j < e; ++j) {
              if (j == i) continue;
              const float *q4 = J->sp + 4 * (size_t)j, *w4 = J->sv + 4 * (size_t)j;
              float rj = J->radius_from_w ? q4[3] : P->particleRadius;
              f3 t = sphere_term(pos, mk3(q4[0], q4[1], q4[2]), vel,
                                 mk3(w4[0], w4[1], w4[2]), ri, rj,
                                 P->attraction, P);
              cf.x = cf.x + t.x; cf.y = cf.y + t.y; cf.z = cf.z + t.z;
            }
          }
          force.x = force.x + cf.x;
          force.y = force.y + cf.y;
          force.z = force.z + cf.z;
        }
    if (J->with_collider) { /* particles_kernel.cu:288 */
      f3 t = sphere_term(pos, mk3(P->colliderPos[0], P->colliderPos[1],
                                  P->colliderPos[2]),
                         vel, mk3(0.0f, 0.0f, 0.0f), ri, P->colliderRadius,
                         0.0f, P);
      force.x = force.x + t.x; force.y = force.y + t.y; force.z = force.z + t.z;
    }
    unsigned o = J->index[i];
    float *nv = J->newVel + 4 * (size_t)o;
    nv[0] = vel.x + force.x;
    nv[1] = vel.y + force.y;
    nv[2] = vel.z + force.z;
    nv[3] = 0.0f;
    if (J->force_out) {
      J->force_out[3 * (size_t)o] = force.x;
      J->force_out[3 * (size_t)o + 1] = force.y;
      J->force_out[3 * (size_t)o + 2] = force.z;
    }
  }
}

/* Double-precision twin of sphere_term. */
static inline void sphere_term64(const double pA[3], const double pB[3],
                                 const double vA[3], const double vB[3],
                                 double rA, double rB, double attraction,
                                 const SimParams *P, double f[3]) {
  double rel[3] = {pB[0] - pA[0], pB[1] - pA[1], pB[2] - pA[2]};
  double dist = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
  double cd = rA + rB;
  f[0] = f[1] = f[2] = 0.0;
  if (dist < cd) {
    double inv = 1.0 / dist;
    double nrm[3] = {rel[0] * inv, rel[1] * inv, rel[2] * inv};
    double rv[3] = {vB[0] - vA[0], vB[1] - vA[1], vB[2] - vA[2]};
    double dn = rv[0] * nrm[0] + rv[1] * nrm[1] + rv[2] * nrm[2];
    double s = -(double)P->spring * (cd - dist);
    for (int k = 0; k < 3; ++k) {
      double tv = rv[k] - nrm[k] * dn;
      f[k] = nrm[k] * s + rv[k] * (double)P->damping +
             tv * (double)P->shear + rel[k] * attraction;
    }
  }
}

static void collide_range64(const collide_job *J) {
  const SimParams *P = J->P;
  for (unsigned i = J->begin; i < J->end; ++i) {
    const float *p4 = J->sp + 4 * (size_t)i, *v4 = J->sv + 4 * (size_t)i;
    double pos[3] = {p4[0], p4[1], p4[2]}, vel[3] = {v4[0], v4[1], v4[2]};
    double ri = J->radius_from_w ? (double)p4[3] : (double)P->particleRadius;
    int g[3];
    grid_pos(P, p4[0], p4[1], p4[2], g);
    double force[3] = {0.0, 0.0, 0.0};
    for (int z = -1; z <= 1; ++z)
      for (int y = -1; y <= 1; ++y)
        for (int x = -1; x <= 1; ++x) {
          unsigned h = grid_hash(P, g[0] + x, g[1] + y, g[2] + z);
          unsigned s = J->cs[h];
          if (s == 0xffffffffu) continue;
          unsigned e = J->ce[h];
          for (unsigned j = s; j < e; ++j) {
            if (j == i) continue;
            const float *q4 = J->sp + 4 * (size_t)j, *w4 = J->sv + 4 * (size_t)j;
            double q[3] = {q4[0], q4[1], q4[2]}, w[3] = {w4[0], w4[1], w4[2]};
            double rj = J->radius_from_w ? (double)q4[3] : (double)P->particleRadius;
            double t[3];
            sphere_term64(pos, q, vel, w, ri, rj, (double)P->attraction, P, t);
            force[0] += t[0]; force[1] += t[1]; force[2] += t[2];
          }
        }
    if (J->with_collider) {
      double c[3] = {P->colliderPos[0], P->colliderPos[1], P->colliderPos[2]};
      double zero[3] = {0.0, 0.0, 0.0}, t[3];
      sphere_term64(pos, c, vel, zero, ri, (double)P->colliderRadius, 0.0, P, t);
      force[0] += t[0]; force[1] += t[1]; force[2] += t[2];
    }
    unsigned o = J->index[i];
    double *nv = J->newVel64 + 4 * (size_t)o;
    nv[0] = vel[0] + force[0];
    nv[1] = vel[1] + force[1];
    nv[2] = vel[2] + force[2];
    nv[3] = 0.0;
  }
}

static void *collide_thread(void *arg) {
  collide_job *J = (collide_job *)arg;
  if (J->newVel64) collide_range64(J); else collide_range(J);
  return NULL;
}

static void run_collide(collide_job base, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if ((unsigned)nthreads > base.n) nthreads = base.n ? (int)base.n : 1;
  if (nthreads == 1) {
    base.begin = 0; base.end = base.n;
    collide_thread(&base);
    return;
  }
  pthread_t th[256];
  collide_job jobs[256];
  unsigned chunk = (base.n + (unsigned)nthreads - 1) / (unsigned)nthreads;
  int started = 0;
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = base;
    jobs[t].begin = (unsigned)t * chunk;
    jobs[t].end = jobs[t].begin + chunk > base.n ? base.n : jobs[t].begin + chunk;
    if (jobs[t].begin >= jobs[t].end) break;
    if (pthread_create(&th[t], NULL, collide_thread, &jobs[t]) != 0) {
      collide_thread(&jobs[t]); /* run inline if no thread is available */
      th[t] = 0;
    }
    started = t + 1;
  }
  for (int t = 0; t < started; ++t)
    if (th[t]) pthread_join(th[t], NULL);
}

void orc_collide(const SimParams *P, float *newVel, float *force_out,
                 const float *sortedPos, const float *sortedVel,
                 const unsigned *index, const unsigned *cellStart,
                 const unsigned *cellEnd, unsigned n, int radius_from_w,
                 int with_collider, int nthreads) {
  collide_job J;
  memset(&J, 0, sizeof(J));
  J.P = P; J.newVel = newVel; J.force_out = force_out; J.sp = sortedPos;
  J.sv = sortedVel; J.index = index; J.cs = cellStart; J.ce = cellEnd;
  J.n = n; J.radius_from_w = radius_from_w; J.with_collider = with_collider;
  run_collide(J, nthreads);
}

void orc_collide_f64(const SimParams *P, double *newVel64,
                     const float *sortedPos, const float *sortedVel,
                     const unsigned *index, const unsigned *cellStart,
                     const unsigned *cellEnd, unsigned n, int radius_from_w,
                     int with_collider, int nthreads) {
  collide_job J;
  memset(&J, 0, sizeof(J));
  J.P = P; J.newVel64 = newVel64; J.sp = sortedPos; J.sv = sortedVel;
  J.index = index; J.cs = cellStart; J.ce = cellEnd; J.n = n;
  J.radius_from_w = radius_from_w; J.with_collider = with_collider;
  run_collide(J, nthreads);
}

/* ---------------------------------------------------------------------- */
/* The same stages on nthreads host threads (the CPU baseline uses every
 * core).  Each gives the single-threaded function's bits: integrate, hash
 * and the reorder's gather are independent per particle; the radix sort
 * keeps its stable order with per-thread digit counts taken over
 * consecutive chunks; a cell's start and end are written by the one
 * element where the sorted hash changes. */
typedef struct {
  int t, nt;
  unsigned n;
  void *ctx;
  void (*fn)(void *ctx, int t, unsigned lo, unsigned hi);
} par_job;

static void *par_thread(void *arg) {
  par_job *J = (par_job *)arg;
  unsigned chunk = (J->n + (unsigned)J->nt - 1) / (unsigned)J->nt;
  unsigned lo = (unsigned)J->t * chunk;
  unsigned hi = lo + chunk < J->n ? lo + chunk : J->n;
  if (lo < hi) J->fn(J->ctx, J->t, lo, hi);
  return NULL;
}

/* fn(ctx, t, lo, hi) for thread t's chunk of [0, n); chunk t is the t-th
 * of nt equal consecutive ranges */
static void parallel_chunks(unsigned n, int nt, void *ctx,
                            void (*fn)(void *ctx, int t, unsigned lo, unsigned hi)) {
  pthread_t th[256];
  par_job jobs[256];
  for (int t = 0; t < nt; ++t) {
    jobs[t].t = t;
    jobs[t].nt = nt;
    jobs[t].n = n;
    jobs[t].ctx = ctx;
    jobs[t].fn = fn;
    th[t] = 0;
    if (t > 0 && pthread_create(&th[t], NULL, par_thread, &jobs[t]) != 0) {
      th[t] = 0;
      par_thread(&jobs[t]);
    }
  }
  par_thread(&jobs[0]);
  for (int t = 1; t < nt; ++t)
    if (th[t]) pthread_join(th[t], NULL);
}

typedef struct {
  const SimParams *P;
  float *pos, *vel, dt;
  int radius_from_w;
  unsigned *hash, *index;
} stage_ctx;

static void integrate_hash_chunk(void *c, int t, unsigned lo, unsigned hi) {
  stage_ctx *S = (stage_ctx *)c;
  (void)t;
  orc_integrate(S->P, S->pos + 4 * (size_t)lo, S->vel + 4 * (size_t)lo, S->dt, hi - lo,
                S->radius_from_w);
  for (unsigned i = lo; i < hi; ++i) {
    int g[3];
    grid_pos(S->P, S->pos[4 * (size_t)i], S->pos[4 * (size_t)i + 1],
             S->pos[4 * (size_t)i + 2], g);
    S->hash[i] = grid_hash(S->P, g[0], g[1], g[2]);
    S->index[i] = i;
  }
}

typedef struct {
  const unsigned *ka, *va;
  unsigned *kb, *vb;
  int shift;
  size_t (*count)[256];  /* per thread: digit counts, then output offsets */
} sort_ctx;

static void sort_count_chunk(void *c, int t, unsigned lo, unsigned hi) {
  sort_ctx *S = (sort_ctx *)c;
  size_t *cnt = S->count[t];
  memset(cnt, 0, 256 * sizeof(size_t));
  for (unsigned i = lo; i < hi; ++i) cnt[(S->ka[i] >> S->shift) & 255u]++;
}

static void sort_scatter_chunk(void *c, int t, unsigned lo, unsigned hi) {
  sort_ctx *S = (sort_ctx *)c;
  size_t *off = S->count[t];
  for (unsigned i = lo; i < hi; ++i) { /* ascending i within the chunk: stable */
    size_t dst = off[(S->ka[i] >> S->shift) & 255u]++;
    S->kb[dst] = S->ka[i];
    S->vb[dst] = S->va[i];
  }
}

static void sort_pairs_par(unsigned *keys, unsigned *vals, unsigned n, int nt) {
  if (n < 2) return;
  unsigned *k2 = (unsigned *)malloc(sizeof(unsigned) * (size_t)n);
  unsigned *v2 = (unsigned *)malloc(sizeof(unsigned) * (size_t)n);
  size_t (*count)[256] = (size_t(*)[256])malloc(sizeof(size_t) * 256 * (size_t)nt);
  unsigned *ka = keys, *va = vals, *kb = k2, *vb = v2;
  for (int shift = 0; shift < 32; shift += 8) {
    sort_ctx S = {ka, va, kb, vb, shift, count};
    parallel_chunks(n, nt, &S, sort_count_chunk);
    size_t total[256];
    memset(total, 0, sizeof(total));
    for (int t = 0; t < nt; ++t)
      for (int d = 0; d < 256; ++d) total[d] += count[t][d];
    int trivial = 0;
    for (int d = 0; d < 256; ++d)
      if (total[d] == n) trivial = 1;
    if (trivial) continue; /* one digit value: the pass is the identity */
    /* digit-major, thread-minor offsets: the stable order of the
     * single-threaded pass */
    size_t run = 0;
    for (int d = 0; d < 256; ++d)
      for (int t = 0; t < nt; ++t) {
        size_t c = count[t][d];
        count[t][d] = run;
        run += c;
      }
    parallel_chunks(n, nt, &S, sort_scatter_chunk);
    unsigned *tmp = ka; ka = kb; kb = tmp;
    tmp = va; va = vb; vb = tmp;
  }
  if (ka != keys) {
    memcpy(keys, ka, sizeof(unsigned) * (size_t)n);
    memcpy(vals, va, sizeof(unsigned) * (size_t)n);
  }
  free(count);
  free(k2);
  free(v2);
}

typedef struct {
  unsigned *cellStart, *cellEnd;
  float *sortedPos, *sortedVel;
  const unsigned *hash, *index;
  const float *oldPos, *oldVel;
  unsigned n, numCells;
} reorder_ctx;

static void reorder_clear_chunk(void *c, int t, unsigned lo, unsigned hi) {
  reorder_ctx *R = (reorder_ctx *)c;
  (void)t;
  memset(R->cellStart + lo, 0xff, sizeof(unsigned) * (size_t)(hi - lo));
}

static void reorder_chunk(void *c, int t, unsigned lo, unsigned hi) {
  reorder_ctx *R = (reorder_ctx *)c;
  (void)t;
  for (unsigned i = lo; i < hi; ++i) {
    unsigned h = R->hash[i];
    if (i == 0 || h != R->hash[i - 1]) {
      R->cellStart[h] = i;
      if (i > 0) R->cellEnd[R->hash[i - 1]] = i;
    }
    if (i == R->n - 1) R->cellEnd[h] = i + 1;
    unsigned s = R->index[i];
    memcpy(R->sortedPos + 4 * (size_t)i, R->oldPos + 4 * (size_t)s, 16);
    memcpy(R->sortedVel + 4 * (size_t)i, R->oldVel + 4 * (size_t)s, 16);
  }
}

void orc_update(const SimParams *P, float dt, float *pos, float *vel,
                float *sortedPos, float *sortedVel, unsigned *hash,
                unsigned *index, unsigned *cellStart, unsigned *cellEnd,
                unsigned n, int radius_from_w, int nthreads) {
  int nt = nthreads < 1 ? 1 : (nthreads > 256 ? 256 : nthreads);
  if ((unsigned)nt > n / 4096u + 1u) nt = (int)(n / 4096u) + 1;  /* small n: fewer */
  if (nt == 1) {
    orc_integrate(P, pos, vel, dt, n, radius_from_w);
    orc_calc_hash(P, hash, index, pos, n);
    orc_sort_pairs(hash, index, n);
    orc_reorder(cellStart, cellEnd, sortedPos, sortedVel, hash, index, pos, vel,
                n, P->numCells);
  } else {
    stage_ctx S = {P, pos, vel, dt, radius_from_w, hash, index};
    parallel_chunks(n, nt, &S, integrate_hash_chunk);
    sort_pairs_par(hash, index, n, nt);
    reorder_ctx R = {cellStart, cellEnd, sortedPos, sortedVel, hash, index,
                     pos, vel, n, P->numCells};
    parallel_chunks(P->numCells, nt, &R, reorder_clear_chunk);
    parallel_chunks(n, nt, &R, reorder_chunk);
  }
  orc_collide(P, vel, NULL, sortedPos, sortedVel, index, cellStart, cellEnd, n,
              radius_from_w, 1, nthreads);
}

/* ---------------------------------------------------------------------- */
/* Distance map. */

static int check_distmap_fused(const orc_distmap *m, float r, float bd, float p[3],
                               float v[3]);

static inline int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

/* vertex coordinate along one axis: vertices_[0] + i*cellSize_ in float
 * (distancemap.cpp:221-223) */
static inline float vcoord(float vmin, int i, float cs) {
  float t = (float)i * cs;
  return vmin + t;
}

void orc_distmap_query(const orc_distmap *m, const float q[3], float *dist,
                       float cp[3]) {
  /* AABB3::isPointInside (aabb3.h:173-181), inclusive faces */
  if (!(m->vmin[0] <= q[0] && q[0] <= m->vmax[0] && m->vmin[1] <= q[1] &&
        q[1] <= m->vmax[1] && m->vmin[2] <= q[2] && q[2] <= m->vmax[2])) {
    *dist = 5.0f;
    return;
  }
  float inv = (float)(1.0 / (double)m->cellSize);
  int c[3];
  for (int k = 0; k < 3; ++k) {
    c[k] = (int)(fabsf(q[k] - m->vmin[k]) * inv);
    c[k] = clampi(c[k], 0, m->cells[k] - 1);
  }
  /* vertexIndices, distancemap.cuh:281-302 */
  int ix = m->cells[0] + 1;
  int islice = (m->cells[0] + 1) * (m->cells[1] + 1);
  int b = c[2] * islice + c[1] * ix + c[0];
  int idx[8] = {b, b + 1, b + ix + 1, b + ix, b + islice, b + islice + 1,
                b + ix + islice + 1, b + ix + islice};
  float x0 = vcoord(m->vmin[0], c[0], m->cellSize);
  float x1 = vcoord(m->vmin[0], c[0] + 1, m->cellSize);
  float y0 = vcoord(m->vmin[1], c[1], m->cellSize);
  float y1 = vcoord(m->vmin[1], c[1] + 1, m->cellSize);
  float z0 = vcoord(m->vmin[2], c[2], m->cellSize);
  float z1 = vcoord(m->vmin[2], c[2] + 1, m->cellSize);
  float xd = (q[0] - x0) / (x1 - x0);
  float yd = (q[1] - y0) / (y1 - y0);
  float zd = (q[2] - z0) / (z1 - z0);
  /* trilinearInterpolateDistance, distancemap.cuh:227-252.  In
   * `d0 * (1.0 - x_d) + d1 * x_d` the first product is double (1.0 is a
   * double literal), the second float * float; the sum is double and is
   * rounded to float on assignment. */
  const float *D = m->distance;
  double wx = 1.0 - (double)xd, wy = 1.0 - (double)yd, wz = 1.0 - (double)zd;
  float c00 = (float)((double)D[idx[0]] * wx + (double)(D[idx[1]] * xd));
  float c10 = (float)((double)D[idx[3]] * wx + (double)(D[idx[2]] * xd));
  float c01 = (float)((double)D[idx[4]] * wx + (double)(D[idx[5]] * xd));
  float c11 = (float)((double)D[idx[7]] * wx + (double)(D[idx[6]] * xd));
  float c0 = (float)((double)c00 * wy + (double)(c10 * yd));
  float c1 = (float)((double)c01 * wy + (double)(c11 * yd));
  *dist = (float)((double)c0 * wz + (double)(c1 * zd));
  /* trilinearInterpolateCP, distancemap.cuh:254-279: Vector3<float> times a
   * float weight (the double weight converted to float). */
  const float *C = m->contactPoints;
  float fwx = (float)wx, fwy = (float)wy, fwz = (float)wz;
  for (int k = 0; k < 3; ++k) {
    float a00 = C[3 * idx[0] + k] * fwx + C[3 * idx[1] + k] * xd;
    float a10 = C[3 * idx[3] + k] * fwx + C[3 * idx[2] + k] * xd;
    float a01 = C[3 * idx[4] + k] * fwx + C[3 * idx[5] + k] * xd;
    float a11 = C[3 * idx[7] + k] * fwx + C[3 * idx[6] + k] * xd;
    float a0 = a00 * fwy + a10 * yd;
    float a1 = a01 * fwy + a11 * yd;
    cp[k] = a0 * fwz + a1 * zd;
  }
}

void orc_check_distmap(const orc_distmap *m, float radius,
                       float boundaryDamping, float pos[3], float vel[3]) {
  float dist = 0.0f, cp[3] = {0.0f, 0.0f, 0.0f};
  orc_distmap_query(m, pos, &dist, cp);
  if (dist < radius) {
    float n0[3] = {pos[0] - cp[0], pos[1] - cp[1], pos[2] - cp[2]};
    /* normalize: v * rsqrtf(dot(v, v)); rsqrtf restated as 1/sqrtf */
    float invLen = 1.0f / sqrtf(n0[0] * n0[0] + n0[1] * n0[1] + n0[2] * n0[2]);
    float n[3] = {n0[0] * invLen, n0[1] * invLen, n0[2] * invLen};
    float pen = radius - dist;
    float extra = (float)(0.1 * (double)radius);
    for (int k = 0; k < 3; ++k) {
      float t = pos[k] + n[k] * pen;
      pos[k] = t + n[k] * extra;
    }
    vel[0] = vel[0] * (0.5f * boundaryDamping);
    vel[1] = vel[1] * (0.5f * boundaryDamping);
    vel[2] = vel[2] * (0.7f * boundaryDamping);
  }
}

void orc_integrate_distmap(const SimParams *P, const orc_distmap *m,
                           float *pos, float *vel, float dt, unsigned n,
                           int radius_from_w) {
  for (unsigned i = 0; i < n; ++i) {
    float *p4 = pos + 4 * (size_t)i, *v4 = vel + 4 * (size_t)i;
    float p[3] = {p4[0], p4[1], p4[2]}, v[3] = {v4[0], v4[1], v4[2]};
    float r = radius_from_w ? p4[3] : P->particleRadius;
    float bd = P->boundaryDamping;
    if (g_gpu_arith) {
      for (int k = 0; k < 3; ++k) v[k] = fmaf(P->gravity[k], dt, v[k]);
      for (int k = 0; k < 3; ++k) v[k] = v[k] * P->globalDamping;
      for (int k = 0; k < 3; ++k) p[k] = fmaf(v[k], dt, p[k]);
    } else {
      for (int k = 0; k < 3; ++k) v[k] = v[k] + P->gravity[k] * dt;
      for (int k = 0; k < 3; ++k) v[k] = v[k] * P->globalDamping;
      for (int k = 0; k < 3; ++k) p[k] = p[k] + v[k] * dt;
    }
    /* d_checkBoundaryDistMap, boundaries.cuh:65-89: the cylinder test uses
     * the position before the map push. */
    float l2 = g_gpu_arith ? fmaf(p[0], p[0], p[1] * p[1])
                           : p[0] * p[0] + p[1] * p[1] + 0.0f * 0.0f;
    float len = sqrtf(l2);
    float px0 = p[0], py0 = p[1];
    if (g_gpu_arith) check_distmap_fused(m, r, bd, p, v);
    else orc_check_distmap(m, r, bd, p, v);
    if (len > 1.0f) {
      float pen = len - 1.0f;
      float invLen = 1.0f / sqrtf(l2);
      float nx = px0 * invLen, ny = py0 * invLen, nz = 0.0f * invLen;
      float s = pen + r;
      if (g_gpu_arith) {
        p[0] = fmaf(-nx, s, p[0]);
        p[1] = fmaf(-ny, s, p[1]);
        p[2] = fmaf(-nz, s, p[2]);
      } else {
        p[0] = p[0] - nx * s;
        p[1] = p[1] - ny * s;
        p[2] = p[2] - nz * s;
      }
      v[0] = v[0] * bd;
      v[1] = v[1] * bd;
    }
    if (p[2] > 10.0f - r) { p[2] = 10.0f - r; v[2] = v[2] * bd; }
    if (p[2] < -1.0f + r) { p[2] = -1.0f + r; v[2] = v[2] * bd; }
    p4[0] = p[0]; p4[1] = p[1]; p4[2] = p[2];
    /* particledem_um.cu:636 stores vel.w = pos.w */
    v4[0] = v[0]; v4[1] = v[1]; v4[2] = v[2]; v4[3] = p4[3];
  }
}

/* ---------------------------------------------------------------------- */
/* Batched scenes.  Each scene of a batch is stepped as one ParticleSystem
 * with its own parameters and its own box [lo, hi] (the reference's box is
 * [-1, 1]^3).  Below, the reference's GPU arithmetic is restated as nvcc
 * builds it: `vel += gravity * deltaTime` and `pos += vel * deltaTime` of
 * particles_kernel.cu:55-59 and particledem_um.cu:625-630 are contracted
 * into fused multiply-adds (fmaf, correctly rounded in C99 as on the GPU). */

/* particles_kernel.cu:39-75 with the faces of the box [lo, hi], in the
 * reference's order (+x, -x, +y, +z, -z, -y). */
static inline void box_faces(float lo[3], float hi[3], float r, float bd,
                             float p[3], float v[3]) {
  if (p[0] > hi[0] - r) { p[0] = hi[0] - r; v[0] = v[0] * bd; }
  if (p[0] < lo[0] + r) { p[0] = lo[0] + r; v[0] = v[0] * bd; }
  if (p[1] > hi[1] - r) { p[1] = hi[1] - r; v[1] = v[1] * bd; }
  if (p[2] > hi[2] - r) { p[2] = hi[2] - r; v[2] = v[2] * bd; }
  if (p[2] < lo[2] + r) { p[2] = lo[2] + r; v[2] = v[2] * bd; }
  if (p[1] < lo[1] + r) { p[1] = lo[1] + r; v[1] = v[1] * bd; }
}

void orc_integrate_box(const SimParams *P, const float lo[3], const float hi[3],
                       float *pos, float *vel, float dt, unsigned n,
                       int radius_from_w) {
  float l[3] = {lo[0], lo[1], lo[2]}, h[3] = {hi[0], hi[1], hi[2]};
  for (unsigned i = 0; i < n; ++i) {
    float *p4 = pos + 4 * (size_t)i, *v4 = vel + 4 * (size_t)i;
    float p[3] = {p4[0], p4[1], p4[2]}, v[3] = {v4[0], v4[1], v4[2]};
    float r = radius_from_w ? p4[3] : P->particleRadius;
    for (int k = 0; k < 3; ++k) v[k] = fmaf(P->gravity[k], dt, v[k]);
    for (int k = 0; k < 3; ++k) v[k] = v[k] * P->globalDamping;
    for (int k = 0; k < 3; ++k) p[k] = fmaf(v[k], dt, p[k]);
    box_faces(l, h, r, P->boundaryDamping, p, v);
    p4[0] = p[0]; p4[1] = p[1]; p4[2] = p[2];
    v4[0] = v[0]; v4[1] = v[1]; v4[2] = v[2];
  }
}

/* distancemap.cuh:154-191 as the GPU build evaluates it: the distance as in
 * orc_distmap_query (its double products are not contracted), each
 * contact-point blend `a * w0 + b * w1` of trilinearInterpolateCP
 * (distancemap.cuh:254-279) as fmaf(a, w0, b * w1). */
static void distmap_query_fused(const orc_distmap *m, const float q[3],
                                float *dist, float cp[3]) {
  orc_distmap_query(m, q, dist, cp);
  if (*dist == 5.0f &&
      !(m->vmin[0] <= q[0] && q[0] <= m->vmax[0] && m->vmin[1] <= q[1] &&
        q[1] <= m->vmax[1] && m->vmin[2] <= q[2] && q[2] <= m->vmax[2]))
    return;
  float inv = (float)(1.0 / (double)m->cellSize);
  int c[3];
  for (int k = 0; k < 3; ++k)
    c[k] = clampi((int)(fabsf(q[k] - m->vmin[k]) * inv), 0, m->cells[k] - 1);
  int ix = m->cells[0] + 1;
  int islice = (m->cells[0] + 1) * (m->cells[1] + 1);
  int b = c[2] * islice + c[1] * ix + c[0];
  int idx[8] = {b, b + 1, b + ix + 1, b + ix, b + islice, b + islice + 1,
                b + ix + islice + 1, b + ix + islice};
  float x0 = vcoord(m->vmin[0], c[0], m->cellSize);
  float x1 = vcoord(m->vmin[0], c[0] + 1, m->cellSize);
  float y0 = vcoord(m->vmin[1], c[1], m->cellSize);
  float y1 = vcoord(m->vmin[1], c[1] + 1, m->cellSize);
  float z0 = vcoord(m->vmin[2], c[2], m->cellSize);
  float z1 = vcoord(m->vmin[2], c[2] + 1, m->cellSize);
  float xd = (q[0] - x0) / (x1 - x0);
  float yd = (q[1] - y0) / (y1 - y0);
  float zd = (q[2] - z0) / (z1 - z0);
  float fwx = (float)(1.0 - (double)xd), fwy = (float)(1.0 - (double)yd);
  float fwz = (float)(1.0 - (double)zd);
  const float *C = m->contactPoints;
  for (int k = 0; k < 3; ++k) {
    float a00 = fmaf(C[3 * idx[0] + k], fwx, C[3 * idx[1] + k] * xd);
    float a10 = fmaf(C[3 * idx[3] + k], fwx, C[3 * idx[2] + k] * xd);
    float a01 = fmaf(C[3 * idx[4] + k], fwx, C[3 * idx[5] + k] * xd);
    float a11 = fmaf(C[3 * idx[7] + k], fwx, C[3 * idx[6] + k] * xd);
    float a0 = fmaf(a00, fwy, a10 * yd);
    float a1 = fmaf(a01, fwy, a11 * yd);
    cp[k] = fmaf(a0, fwz, a1 * zd);
  }
}

/* checkDistMap (boundaries.cuh:38-63) as the GPU build evaluates it: the
 * fused contact-point blend, the normal's squared length and the two
 * position updates as fmaf; rsqrtf restated as 1/sqrtf (the GPU's rsqrtf is
 * within 2 ulp of it).  Returns 1 when the map pushed the particle. */
static int check_distmap_fused(const orc_distmap *m, float r, float bd, float p[3],
                               float v[3]) {
  float dist = 0.0f, cp[3] = {0.0f, 0.0f, 0.0f};
  distmap_query_fused(m, p, &dist, cp);
  if (!(dist < r)) return 0;
  float n0[3] = {p[0] - cp[0], p[1] - cp[1], p[2] - cp[2]};
  float dd = fmaf(n0[0], n0[0], fmaf(n0[1], n0[1], n0[2] * n0[2]));
  float invLen = 1.0f / sqrtf(dd);
  float nn[3] = {n0[0] * invLen, n0[1] * invLen, n0[2] * invLen};
  float pen = r - dist;
  float extra = (float)(0.1 * (double)r);
  for (int k = 0; k < 3; ++k) p[k] = fmaf(nn[k], pen, p[k]);
  for (int k = 0; k < 3; ++k) p[k] = fmaf(nn[k], extra, p[k]);
  v[0] = v[0] * (0.5f * bd);
  v[1] = v[1] * (0.5f * bd);
  v[2] = v[2] * (0.7f * bd);
  return 1;
}

void orc_batch_obstacle_integrate(const SimParams *P, const float lo[3],
                                  const float hi[3], const orc_distmap *m,
                                  float *pos, float *vel, float dt, unsigned n,
                                  int radius_from_w, unsigned *contacts) {
  float l[3] = {lo[0], lo[1], lo[2]}, h[3] = {hi[0], hi[1], hi[2]};
  unsigned nc = 0;
  for (unsigned i = 0; i < n; ++i) {
    float *p4 = pos + 4 * (size_t)i, *v4 = vel + 4 * (size_t)i;
    float p[3] = {p4[0], p4[1], p4[2]}, v[3] = {v4[0], v4[1], v4[2]};
    float r = radius_from_w ? p4[3] : P->particleRadius;
    float bd = P->boundaryDamping;
    /* particledem_um.cu:625-630 */
    for (int k = 0; k < 3; ++k) v[k] = fmaf(P->gravity[k], dt, v[k]);
    for (int k = 0; k < 3; ++k) v[k] = v[k] * P->globalDamping;
    for (int k = 0; k < 3; ++k) p[k] = fmaf(v[k], dt, p[k]);
    if (m) nc += (unsigned)check_distmap_fused(m, r, bd, p, v); /* boundaries.cuh:38-63 */
    box_faces(l, h, r, bd, p, v);
    p4[0] = p[0]; p4[1] = p[1]; p4[2] = p[2];
    v4[0] = v[0]; v4[1] = v[1]; v4[2] = v[2];
  }
  if (contacts) *contacts = nc;
}
