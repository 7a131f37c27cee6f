/*
 * fcdem.h -- C-ABI of the GB300 (sm_103a) particle-DEM step.
 *
 * The first block of entry points has exactly the names, argument lists and
 * meaning of FullC0ntact's particle-system C interface
 * (cuda_addon/particleSystem.cuh:12-63, implemented in
 * cuda_addon/particleSystem.cu:36-272), so host code written against that
 * header links against libfcdem.so unchanged.  Pointers are DEVICE pointers;
 * positions and velocities are float4 per particle (x, y, z, w), 16 bytes.
 *
 * Behaviour kept from the reference:
 *   - every stage is issued in order on one CUDA stream (the legacy default
 *     stream unless fcdemSetStream() names another one);
 *   - calcHash writes index[i] = i; sortParticles is a stable ascending sort of
 *     (hash, index) pairs; reorderDataAndFindCellStart sets cellStart of empty
 *     cells to 0xffffffff and leaves cellEnd of empty cells untouched;
 *   - collide writes newVel[index[i]] = (v + F, 0) where F is the summed
 *     spring/dashpot/shear/attraction term over the 27 wrapped neighbour cells
 *     plus the collider sphere term.
 * Differences:
 *   - no entry point calls exit(); failures are recorded and returned by
 *     fcdemGetLastError();
 *   - the OpenGL interop entry points exist only as stubs that record
 *     FCDEM_ERR_UNSUPPORTED (no graphics stack on the target);
 *   - extensions are prefixed fcdem* and documented below.
 */
#ifndef FCDEM_H
#define FCDEM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------- */
/* SimParams: 104 bytes, 4-byte aligned, field order and offsets of
 * cuda_addon/particles_kernel.cuh:27-48.  When the reference header has been
 * included first (its guard is PARTICLES_KERNEL_H) its definition is used. */
#ifndef PARTICLES_KERNEL_H
typedef unsigned int uint;
typedef struct SimParams {
  float colliderPos[3];        /*   0 */
  float colliderRadius;        /*  12 */
  float gravity[3];            /*  16 */
  float globalDamping;         /*  28 */
  float particleRadius;        /*  32 */
  unsigned int gridSize[3];    /*  36  each a power of two */
  unsigned int numCells;       /*  48 */
  float worldOrigin[3];        /*  52 */
  float cellSize[3];           /*  64 */
  unsigned int numBodies;      /*  76 */
  unsigned int maxParticlesPerCell; /* 80  unused, as in the reference */
  float spring;                /*  84 */
  float damping;               /*  88 */
  float shear;                 /*  92 */
  float attraction;            /*  96 */
  float boundaryDamping;       /* 100 */
} SimParams;
#endif

struct cudaGraphicsResource;

/* ---------------------------------------------------------------------- */
/* Support calls (particleSystem.cuh:14-26). */

/* particleSystem.cu:39-63: selects a device.  "-device=N" in argv picks N,
 * otherwise device 0 (the GB300 build targets one GPU per process). */
void cudaInit(int argc, char **argv);
/* particleSystem.cu:65-68, with the argument type of the reference's header
 * (particleSystem.cuh:16 declares int; its implementation takes size_t, a
 * mismatch the reference's callers never see): size is a byte count below
 * 2^31, a negative size records FCDEM_ERR_INVALID_VALUE. */
void allocateArray(void **devPtr, int size);
/* particleSystem.cu:70-73 */
void freeArray(void *devPtr);
/* particleSystem.cu:75-78: waits for all work issued by this library. */
void threadSync(void);
/* particleSystem.cu:111-121: a non-null GL resource records
 * FCDEM_ERR_UNSUPPORTED and copies nothing. */
void copyArrayFromDevice(void *host, const void *device,
                         struct cudaGraphicsResource **cuda_vbo_resource,
                         int size);
/* particleSystem.cu:80-83 */
void copyArrayToDevice(void *device, const void *host, int offset, int size);
/* particleSystem.cu:85-109: OpenGL interop.  Stubs: record
 * FCDEM_ERR_UNSUPPORTED; map returns NULL. */
void registerGLBufferObject(uint vbo, struct cudaGraphicsResource **cuda_vbo_resource);
void unregisterGLBufferObject(struct cudaGraphicsResource *cuda_vbo_resource);
void *mapGLBufferObject(struct cudaGraphicsResource **cuda_vbo_resource);
void unmapGLBufferObject(struct cudaGraphicsResource *cuda_vbo_resource);

/* ---------------------------------------------------------------------- */
/* The five stages (particleSystem.cuh:29-61). */

/* particleSystem.cu:123-127: copies the parameter block; every later launch
 * on this device uses this copy until the next call. */
void setParameters(SimParams *hostParams);

/* particleSystem.cu:141-153 + particles_kernel.cu:39-75:
 * v += g*dt; v *= globalDamping; p += v*dt; clamp to [-1+r, 1-r] per axis
 * with v_axis *= boundaryDamping on contact.  In place. */
void integrateSystem(float *pos, float *vel, float deltaTime, uint numParticles);

/* particleSystem.cu:165-181 + particles_kernel.cu:78-115:
 * hash[i] = wrapped linear cell id of pos[i], index[i] = i. */
void calcHash(uint *gridParticleHash, uint *gridParticleIndex, float *pos,
              int numParticles);

/* particleSystem.cu:265-270: stable ascending sort of (hash, index) in place.
 * Keys are expected below 2^ceil(log2(numCells)) of the current parameters;
 * a larger key records FCDEM_ERR_KEY_RANGE. */
void sortParticles(uint *dGridParticleHash, uint *dGridParticleIndex,
                   uint numParticles);

/* No counterpart in the reference.  The same sort as sortParticles, for
 * callers that must not have the library allocate device memory: hosts whose
 * own pool owns all device memory and forbid hidden allocations, and loops
 * run near the memory limit, where an allocation in the middle of a step can
 * fail.  sortParticles allocates its scratch on first use; this entry point
 * allocates nothing and uses a fixed ~17 MB scratch array in the library's
 * static device memory, present on every GPU that loads the library until
 * the process exits.
 *   - At most 1,048,576 particles; more records FCDEM_ERR_INVALID_VALUE and
 *     leaves the arrays untouched.
 *   - Key width: that of the numCells last given to setParameters on this
 *     device, all 32 bits before any setParameters.
 *   - Its first call on a device looks up that array's device address (with
 *     the device current) and clears the sort's status word in it; make that
 *     first call before any stream capture.
 *   - Every call shares the one array: calls that overlap on the GPU (other
 *     streams, other host threads) race and corrupt each other's results.
 *     Issue them in order on one stream.
 *   - Device-side errors (a key above the key width, a bounded wait that ran
 *     out) are kept in that array's status word until fcdemGetLastError
 *     reads them. */
void fcdemSortParticlesNoAlloc(uint *dGridParticleHash, uint *dGridParticleIndex,
                               uint numParticles);

/* particleSystem.cu:183-222 + particles_kernel.cu:119-182 */
void reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd,
                                 float *sortedPos, float *sortedVel,
                                 uint *gridParticleHash, uint *gridParticleIndex,
                                 float *oldPos, float *oldVel,
                                 uint numParticles, uint numCells);

/* particleSystem.cu:224-262 + particles_kernel.cu:185-293 */
void collide(float *newVel, float *sortedPos, float *sortedVel,
             uint *gridParticleIndex, uint *cellStart, uint *cellEnd,
             uint numParticles, uint numCells);

/* ---------------------------------------------------------------------- */
/* Extensions (no counterpart in particleSystem.cuh). */

#define FCDEM_SUCCESS               0
#define FCDEM_ERR_INVALID_VALUE     1  /* bad size, null pointer, bad grid   */
#define FCDEM_ERR_CUDA              2  /* a CUDA runtime call failed          */
#define FCDEM_ERR_NO_PARAMS         3  /* a stage ran before setParameters   */
#define FCDEM_ERR_UNSUPPORTED       4  /* OpenGL interop                      */
#define FCDEM_ERR_DEVICE_TIMEOUT    5  /* a bounded device-side wait expired  */
#define FCDEM_ERR_KEY_RANGE         6  /* sort key above the grid's key width */
#define FCDEM_ERR_ALLOC             7  /* device scratch allocation failed    */
#define FCDEM_ERR_RADIUS_BOUND      8  /* a radius above particleRadius (w mode) */
#define FCDEM_ERR_CELL_OVERFLOW     9  /* fcdemUpdate: large-cell list overflowed (internal) */

/* Returns and clears the first error recorded since the last call.  It
 * synchronises the library stream so that device-side status words (bounded
 * waits, key-range checks) are included. */
int fcdemGetLastError(void);
const char *fcdemGetErrorString(int code);

/* All later calls on this host thread's device issue their work on `stream`
 * (a cudaStream_t; NULL = legacy default stream). */
void fcdemSetStream(void *stream);

/* 0 (default): every particle has radius SimParams.particleRadius, exactly as
 * the reference.  1: the radius of particle i is pos[i].w (polydisperse
 * scenes); collide uses radiusA = r_i, radiusB = r_j, which
 * collideSpheres(particles_kernel.cu:185-218) accepts but collideCell never
 * passes, and integrate clamps with r_i.  In this mode particleRadius must be
 * an upper bound of every radius (collide culls cells with it); a larger
 * radius records FCDEM_ERR_RADIUS_BOUND. */
void fcdemSetRadiusMode(int radiusFromW);

/* Cell culling in collide (default on): neighbour cells whose box is farther
 * than the largest contact distance are not scanned.  Results are identical
 * either way; the switch exists to measure and test that. */
void fcdemSetCellCulling(int on);

/* Crowded-neighbourhood path in collide (default on): particles whose 27
 * neighbour cells hold more than a limit (fcdemSetCrowdLimit) are computed
 * by a second kernel, one warp per group of up to 32 members of a cell.
 * Results are identical either way; the switch exists to measure and test
 * that. */
void fcdemSetCrowdPath(int on);
/* Neighbourhood size above which the crowded path takes a particle
 * (0: the default, 512). */
void fcdemSetCrowdLimit(uint limit);

/* Cell-key order (no counterpart in the reference; default 0, the
 * reference's linear hash z*gy*gx + y*gx + x).  1: Morton order -- the cell
 * key of every stage (calcHash, the sort, the cell tables, collide,
 * fcdemUpdate, fcdemUM_update) is the 3-D Morton code of the wrapped cell
 * coordinates, so cells near in space are near in the sorted arrays.
 * Needs a cubic power-of-two grid of at most 1024 cells a side (other grids
 * keep the linear order).  The members of each cell and their order are the
 * same as in linear order, so positions, velocities and forces are
 * identical; hash[] and the cellStart/cellEnd tables are indexed by the
 * Morton key instead. */
void fcdemSetCellOrder(int morton);

/* Library version string. */
const char *fcdemVersion(void);

/* `steps` consecutive ParticleSystem::update calls
 * (particleSystem.cpp:222-284) in one call.  The stages are fused: the first
 * integrate with its calcHash, and every collide except the last with the
 * next update's integrate and calcHash.  On return pos, vel and every work
 * array hold what `steps` reference updates leave in them (cellEnd of empty
 * cells aside, which the reference leaves stale too). */
void fcdemUpdate(float *pos, float *vel, float *sortedPos, float *sortedVel,
                 uint *gridParticleHash, uint *gridParticleIndex,
                 uint *cellStart, uint *cellEnd, float deltaTime,
                 uint numParticles, uint numCells, uint steps);

/* Collide kernel selection: -1 (default) automatic, 0 the global-read
 * kernel, 1 the shared-memory tiled kernel.  Both give identical results. */
void fcdemSetCollidePath(int path);

/* Test hook: the number of look-back rounds a tile of the radix sort
 * (sortParticles, fcdemSortParticlesNoAlloc) may wait for its predecessors
 * before it gives up, records FCDEM_ERR_DEVICE_TIMEOUT and finishes with the
 * prefix it has (a wrong order, every write still inside the arrays).
 * 0: no waiting at all; negative: the default, 2^22 rounds. */
void fcdemSetSortWaitLimit(int rounds);

/* Sort tuning.  The counting passes of the sort come in several block
 * shapes (threads x keys per thread); results are identical.
 * fcdemAutotuneSort times each on numParticles uniform keys below numCells
 * (allocating temporary device memory), keeps the fastest for that size
 * class (power-of-two bucket of numParticles) and returns its index (-1 on
 * error); *bestMs receives its time.  fcdemSetSortConfig forces one
 * (-1 = default) and returns the number of configurations. */
int fcdemAutotuneSort(unsigned numParticles, unsigned numCells, float *bestMs);
int fcdemSetSortConfig(unsigned numParticles, int config);

/* Collide tuning.  A collide configuration is a crowd limit (256, 384, 512,
 * 768 or 1024 neighbourhood members; fcdemSetCrowdLimit), the CTAs per SM of
 * the crowded-neighbourhood kernel's persistent grid (2, 4 or 8) and whether
 * the per-particle kernel copies short neighbour rows to shared memory;
 * results are identical for every one.  fcdemAutotuneCollide times one
 * fcdemUpdate step from the caller's state (the arguments of fcdemUpdate)
 * under each configuration, keeps the fastest -- the default unless another
 * is at least 2% faster -- and returns its index (-1 on error); *bestMs
 * receives its step time.  pos and vel are put back as they
 * were (a temporary device copy); the work arrays hold one step's values.
 * fcdemSetCollideConfig forces one (-1: the default, 512 / 4 / staged) and
 * returns the number of configurations; fcdemGetCollideConfig describes
 * configuration `config` (returns 0, or -1 for an index out of range). */
int fcdemAutotuneCollide(float *pos, float *vel, float *sortedPos, float *sortedVel,
                         uint *gridParticleHash, uint *gridParticleIndex, uint *cellStart,
                         uint *cellEnd, float deltaTime, uint numParticles, uint numCells,
                         float *bestMs);
int fcdemSetCollideConfig(int config);
int fcdemGetCollideConfig(int config, uint *crowdLimit, uint *ctasPerSm, int *stageRows);

/* Number of kernels this library has launched in this process. */
unsigned long long fcdemGetLaunchCount(void);

/* Stage timing of fcdemUpdate.  With profiling on, fcdemUpdate records a CUDA
 * event pair around each stage on its stream.  fcdemGetStageTimes
 * synchronises, adds the elapsed times of the recorded pairs to per-stage
 * totals, writes min(maxStages, FCDEM_NUM_STAGES) totals in milliseconds and
 * the number of timed launches of each stage, and returns FCDEM_NUM_STAGES.
 * Stages: 0 integrate+hash, 1 sort, 2 cell-table fill, 3 reorder,
 * 4 collide.  fcdemSetProfiling(0/1) also clears the totals. */
#define FCDEM_NUM_STAGES 5
void fcdemSetProfiling(int on);
int fcdemGetStageTimes(float *ms, unsigned *launches, int maxStages);

/* fcdemUpdate's sort: 1 (default) a counting sort over the cells with a
 * stable within-cell fix-up fused with the reorder gather; 0 the radix sort,
 * cell-table fill and reorder of the stage functions.  Results are identical. */
void fcdemSetUpdatePipeline(int pipeline);

/* ---------------------------------------------------------------------- */
/* Distance maps (inshape3dcore/grid/distancemap.h:42-57, the GPU copy of
 * cuda_addon/distancemap.cuh:6-116).  A map is a lattice of
 * (cells[0]+1) x (cells[1]+1) x (cells[2]+1) vertices at vmin + i*cellSize
 * holding a signed distance and the closest surface point; vertex (i,j,k)
 * is entry k*(cx+1)*(cy+1) + j*(cx+1) + i. */
typedef struct fcdemDistanceMap fcdemDistanceMap;

/* Uploads a map given in the reference's host layout (distance[V],
 * contactPoints[3V]); NULL arrays leave the vertices zero.  The device copy
 * packs (distance, cp.x, cp.y, cp.z) per vertex, replacing
 * DistanceMap<float,gpu>::transferData (distancemap.cuh:50-95). */
fcdemDistanceMap *fcdemDistMapCreate(const float *distance, const float *contactPoints,
                                     const float vmin[3], const float vmax[3],
                                     float cellSize, const int cells[3]);
/* A map of the torus around the z axis with major radius R and tube radius
 * r, evaluated exactly at each vertex on the GPU: cellsPerAxis cubic cells
 * across x and y over +-(R + r + margin), z rounded up to whole cells over
 * +-(r + margin) (the cubic-cell rule of distancemap.cpp:180-229). */
fcdemDistanceMap *fcdemDistMapTorus(float majorRadius, float tubeRadius, int cellsPerAxis,
                                    float margin);
/* A map of a box with half-extents halfExtents whose edges and corners are
 * rounded with radius `rounding`, centred at the origin: cubic cells, the
 * largest axis cut into cellsPerAxis cells over +-(h + margin).  Exact
 * signed distance and closest point at every vertex. */
fcdemDistanceMap *fcdemDistMapRoundedBox(const float halfExtents[3], float rounding,
                                         int cellsPerAxis, float margin);
/* A map of a closed, outward-oriented triangle mesh (host arrays: xyz per
 * vertex, three vertex indices per triangle), computed on the GPU: at every
 * vertex the distance to the closest point of the mesh, negative inside (by
 * the generalized winding number), and that closest point as the contact
 * point -- what the reference's CGAL builder stores
 * (distancegridcgal.hpp:36-69).  Cubic cells over the mesh box plus the
 * margin, the largest axis cut into cellsPerAxis cells.  Synchronises. */
fcdemDistanceMap *fcdemDistMapFromMesh(const float *vertices3, uint numVertices,
                                       const uint *triangles3, uint numTriangles,
                                       int cellsPerAxis, float margin);
void fcdemDistMapDestroy(fcdemDistanceMap *map);
void fcdemDistMapGeometry(const fcdemDistanceMap *map, float vmin[3], float vmax[3],
                          float *cellSize, int cells[3]);
/* Copies the packed vertices (4 floats each) to host memory. */
void fcdemDistMapVertices(const fcdemDistanceMap *map, float *vertices4);
/* DistanceMap<float,gpu>::queryMap (distancemap.cuh:154-191) for n device
 * points (4 floats each): trilinear distance (5.0 outside the box) and, if
 * cp4 is not NULL, contact point.  A query on the upper face uses the last
 * cell (the reference reads one vertex past the row there). */
void fcdemDistMapQuery(const fcdemDistanceMap *map, const float *queries4, unsigned n,
                       float *dist, float *cp4);

/* particledem_um entry points (cuda_addon/particledem_um.cuh:11-27), with the
 * work arrays as arguments instead of the file's global world and grid.
 *
 * particledem_um.cu:604-638 + boundaries.cuh:65-89: integrate, then the
 * distance-map contact (map may be NULL: none), the r = 1 cylinder around z
 * and the z planes -1 and 10; vel.w receives pos.w as in the reference. */
void fcdemUM_integrateSystem(float *pos, float *vel, float deltaTime, uint numParticles,
                             const fcdemDistanceMap *map);
/* particledem_um.cu:457-602 (evalForces): collide without the collider
 * sphere, newVel[index[i]] = (v + F, 0) and force[index[i]] = F (3 floats). */
void fcdemUM_evalForces(float *newVel, float *force, float *sortedPos, float *sortedVel,
                        uint *gridParticleIndex, uint *cellStart, uint *cellEnd,
                        uint numParticles, uint numCells);
/* particledem_um.cu:442-454: as reorderDataAndFindCellStart, with cellEnd
 * reset to 0xffffffff first as well. */
void fcdemUM_reorderDataAndFindCellStart(uint *cellStart, uint *cellEnd, float *sortedPos,
                                         float *sortedVel, uint *gridParticleHash,
                                         uint *gridParticleIndex, float *oldPos, float *oldVel,
                                         uint numParticles, uint numCells);

/* A rigid particle cluster, the fields of i3d::Rbody<float>
 * (cuda_addon/rbody.hpp:10-22) in their order: member count, up to three
 * member particle indices, centre of mass, velocity. */
typedef struct fcdemRigidBody {
  int numParticles;
  int indices[3];
  float com[3];
  float vel[3];
} fcdemRigidBody;

/* particledem_um.cu:640-718 (d_integrateRigidBody): per body (device
 * array), v += g dt, v *= globalDamping; com.z += v.z dt and vel.z = v.z are
 * stored (the reference stores only z); each member particle's position
 * moves by v dt (w = 1).  Members are the body's own indices (the reference
 * hard-codes particles 0..2 for body 0 and 3..5 for the others, which is the
 * same for its two three-particle bodies). */
void fcdemUM_integrateRigidBodies(fcdemRigidBody *bodies, uint numBodies, float *pos,
                                  uint numParticles, float deltaTime);

/* ---------------------------------------------------------------------- */
/* Neural signed-distance field of an obstacle (no counterpart in the
 * reference).  A small MLP -- inputs (x, y, z) normalised as
 * (x - shift) * scale, optionally a one-hot shape code, `hiddenLayers` SiLU
 * layers of width `hidden` (64 or 128), one linear output times outScale --
 * predicts the distance the map query returns.  Trained on the GPU (FP32
 * forward/backward kernels, Adam) on samples of a distance map; inference
 * runs with BF16 weights and activations on the tensor cores (FP32
 * accumulate).  In the culled boundary integrate the exact map query stays
 * the fallback inside the skin band. */
typedef struct fcdemSdfNet fcdemSdfNet;

/* inputs: 3 + number of shape codes (at most 16); hidden: 64 or 128;
 * hiddenLayers: 2 or 3.  Weights uniform in +-sqrt(6 / fan_in), biases 0. */
fcdemSdfNet *fcdemSdfCreate(int inputs, int hidden, int hiddenLayers,
                            unsigned long long seed);
void fcdemSdfDestroy(fcdemSdfNet *net);
uint fcdemSdfNumParams(const fcdemSdfNet *net);
/* FP32 parameter vector (host): W0 [hidden][inputs], b0, per further hidden
 * layer W [hidden][hidden], b, then wOut [hidden], bOut; row-major [out][in]. */
void fcdemSdfGetParams(const fcdemSdfNet *net, float *host);
void fcdemSdfSetParams(fcdemSdfNet *net, const float *host);
void fcdemSdfSetNormalization(fcdemSdfNet *net, const float shift[3], const float scale[3],
                              float outScale);
void fcdemSdfGetNormalization(const fcdemSdfNet *net, float shift[3], float scale[3],
                              float *outScale);
/* n training samples (device float4: x, y, z, map distance) in the map box:
 * the first nearFraction * n drawn until |distance| < band, the others
 * uniform.  shapes (device int[n], optional) receives `shape`. */
void fcdemSdfSamples(const fcdemDistanceMap *map, int shape, uint n, float nearFraction,
                     float band, unsigned long long seed, float *samples4, int *shapes);
/* Loss sum_s w_s (y_s - d_s / outScale)^2 / n, w_s = 10 when |d_s| < band
 * else 1, and its gradient (host float[numParams], optional) for the device
 * samples. */
float fcdemSdfGradient(fcdemSdfNet *net, const float *samples4, const int *shapes, uint n,
                       float band, float *gradHost);
/* Adam over `epochs` passes of mini-batches of `batch` samples, learning rate
 * lr with cosine decay to lr / 20.  Returns the last epoch's mean loss. */
float fcdemSdfTrainSamples(fcdemSdfNet *net, const float *samples4, const int *shapes, uint n,
                           uint epochs, uint batch, float lr, float band);
/* Distance predictions d[n] at device points (float4, w ignored): FP32 on
 * the CUDA cores, or BF16 on the tensor cores. */
void fcdemSdfEvalF32(fcdemSdfNet *net, const float *points4, const int *shapes, uint n,
                     float *d);
void fcdemSdfInfer(fcdemSdfNet *net, const float *points4, const int *shapes, uint n,
                   float *d);
/* How the network culls the map query (fcdemUM_update, fcdemUM_integrateSystemSdf,
 * batch obstacles).  lipschitz 0 (the default): per particle, the network
 * runs on every 128-slot tile with a particle in the map box and a particle
 * is queried when its prediction is at most `skin`.  lipschitz > 0: per tile
 * of 32 slots, the network runs once, at the centre c of the box bounding
 * the tile's particles in the map box (rho: c to the box's corners), and the
 * tile's queries are skipped when pred(c) - lipschitz * rho > skin; otherwise
 * each of its particles in the map box is queried.  `lipschitz` must bound
 * the network's prediction's Lipschitz constant (sdf.calibrate_lipschitz
 * measures one); then a tile is skipped only where the per-particle rule
 * would skip each of its particles.  A batch replayed from a graph records
 * again after a change. */
void fcdemSdfSetTileCulling(fcdemSdfNet *net, float lipschitz);
/* `steps` unified-memory DEM steps (CollisionPipeline<dem_gpu_unified>::
 * startPipeline, dempipeline.hpp:113-120: calcHash, sortParticles,
 * reorderDataAndFindCellStart, evalForces, integrateSystem with the map
 * boundary) in one call.  force (float3[n], optional) receives evalForces'
 * force of the last step.  With net, the integrate culls the map query as
 * fcdemUM_integrateSystemSdf.  On return every array holds what the staged
 * calls leave (cellEnd of empty cells aside). */
void fcdemUM_update(float *pos, float *vel, float *force, float *sortedPos, float *sortedVel,
                    uint *hash, uint *index, uint *cellStart, uint *cellEnd, float deltaTime,
                    uint numParticles, uint numCells, uint steps, const fcdemDistanceMap *map,
                    fcdemSdfNet *net, float skin, uint *exactQueries);

/* fcdemUM_integrateSystem with the map query made only where the particle is
 * in the map box and the network predicts a distance of at most `skin`;
 * exactQueries (device counter, optional) is incremented per exact query. */
void fcdemUM_integrateSystemSdf(float *pos, float *vel, float deltaTime, uint numParticles,
                                const fcdemDistanceMap *map, fcdemSdfNet *net, float skin,
                                uint *exactQueries);

/* ---------------------------------------------------------------------- */
/* Batches: many independent scenes stepped together (no counterpart in the
 * reference, which steps one ParticleSystem at a time).  Every scene has its
 * own SimParams (grid, cell size, origin, contact parameters), its own box
 * [boxLo, boxHi] that integrate clamps to (the reference's box is [-1,1]^3),
 * and numParticles particles; the particle arrays of a batch are the scenes'
 * arrays concatenated in scene order (4 floats per particle, device memory). */
typedef struct fcdemBatchScene {
  SimParams params;
  float boxLo[3], boxHi[3];
  uint numParticles;
} fcdemBatchScene;
typedef struct fcdemBatch fcdemBatch;

/* radiusFromW applies to every scene (fcdemSetRadiusMode). */
fcdemBatch *fcdemBatchCreate(const fcdemBatchScene *scenes, uint numScenes, int radiusFromW);
void fcdemBatchDestroy(fcdemBatch *batch);
/* Obstacles (no counterpart in the reference): scene s gets the distance map
 * maps[sceneShape[s]] (-1: none), centred in its coordinates.  Each integrate
 * of the batch then applies checkDistMap (boundaries.cuh:38-63) between the
 * velocity/position update and the box clamp.  With net, the map query is
 * culled where the network (shape code = sceneShape[s]) predicts a distance
 * above `skin`.  The maps and the network must outlive their use; numMaps 0
 * removes the obstacles.  Synchronises. */
void fcdemBatchSetObstacles(fcdemBatch *batch, const fcdemDistanceMap *const *maps,
                            uint numMaps, const int *sceneShape, fcdemSdfNet *net, float skin);
/* Exact map queries made by the batch's integrates since the last reset
 * (synchronises); reset != 0 clears the count. */
unsigned long long fcdemBatchExactQueries(fcdemBatch *batch, int reset);
uint fcdemBatchNumParticles(const fcdemBatch *batch);
uint fcdemBatchNumCells(const fcdemBatch *batch);
/* `steps` updates of every scene, each stage one launch over all particles.
 * useGraph: the sequence is recorded as a CUDA graph on the first call (and
 * again when pos, vel, deltaTime or steps change, or the obstacles' network
 * has been trained or given new parameters or normalisation since) and
 * replayed.  The result equals `steps` ParticleSystem-style updates of each
 * scene on its own (with the scene's box). */
void fcdemBatchUpdate(fcdemBatch *batch, float *pos, float *vel, float deltaTime, uint steps,
                      int useGraph);

/* Particle output for ParaView, the format of CVtkWriter::WriteGPUParticleFile
 * (inshape3dcore/postprocessing/vtkwriter.cpp:3399-3452): legacy ASCII
 * UNSTRUCTURED_GRID with the positions of n particles (host array, 4 floats
 * each), a "radius" scalar (pos.w when radiusFromW, else `radius`; the
 * reference writes 1/64 for every particle) and a "myid" scalar.  When vel4 is
 * not NULL a "velocity" vector is added.  Returns 0, or FCDEM_ERR_INVALID_VALUE
 * when the file cannot be written. */
int fcdemWriteVtkParticles(const char *path, const float *pos4, const float *vel4,
                           uint n, float radius, int radiusFromW);

/* CVtkWriter::WriteGPUParticleFile(pPos, strFileName)
 * (inshape3dcore/postprocessing/vtkwriter.cpp:3399-3452) byte for byte: the
 * reference's header lines, the n positions of pos4 (4 floats each, as the
 * reference's pPos vector), a radius of 1/64 for every particle and the
 * "myid" scalar.  Where the reference prints a message and exits the
 * process when the file cannot be opened, this returns
 * FCDEM_ERR_INVALID_VALUE. */
int fcdemWriteGPUParticleFile(const float *pos4, uint n, const char *path);

/* ---------------------------------------------------------------------- */
/* Scene generators (host memory, 4 floats per particle).  Deterministic for
 * a given seed on every platform. */

/* Jittered lattice of ParticleSystem::initGrid (particleSystem.cpp:380-402):
 * side s = ceil(n^(1/3)) particles, pos = spacing*(x,y,z) + radius - 1 +
 * U(-jitter, jitter), w = 1; velocities U(-velRange, velRange), w = 0. */
void fcdemSceneLattice(float *pos4, float *vel4, uint n, float radius,
                       float spacing, float jitter, float velRange,
                       unsigned long long seed);

/* Random sequential packing of n spheres with the given radii (host array)
 * inside [boxMin, boxMax]; the radii are placed largest first within z slabs.
 * pos.w = radius.  Returns the number placed. */
uint fcdemScenePackRadii(float *pos4, float *vel4, uint n, const float *radii,
                         const float boxMin[3], const float boxMax[3], float velRange,
                         unsigned long long seed, uint maxAttempts);

/* Random sequential packing of n spheres with lognormal radii (median rMedian,
 * log-sigma sigma, clipped to rMax) inside [boxMin, boxMax]; pos.w = radius.
 * Radii are placed largest first; a sphere that finds no free spot after
 * maxAttempts tries ends the packing.  Returns the number placed. */
uint fcdemScenePack(float *pos4, float *vel4, uint n, const float boxMin[3],
                    const float boxMax[3], float rMedian, float sigma, float rMax,
                    float velRange, unsigned long long seed, uint maxAttempts);

#ifdef __cplusplus
}
#endif

#endif /* FCDEM_H */
