/*
 * picurv_shim.c -- PICurv's particle-path functions with the reference's own signatures
 * (walkingsearch.h, ParticleSwarm.h, ParticleMotion.h, interpolation.h), implemented over the
 * C ABI of include/fdf_gb300.h.  A PICurv build compiles this file in place of the same functions
 * of walkingsearch.c, ParticleSwarm.c, ParticleMotion.c and interpolation.c and links
 * libfdf_gb300.so: the host code keeps its UserCtx, DMDA vectors and DMSwarm, and the walk, the
 * interpolation and the scatter run on the GPU.
 *
 * What runs where:
 *   - the per-cell and per-particle arithmetic (GetCellCharacteristicSize,
 *     ComputeSignedDistanceToPlane, CalculateDistancesToCellFaces, DeterminePointPosition,
 *     EvaluateParticlePosition, UpdateCellIndicesBasedOnDistancesTEST, UpdateParticleWeights,
 *     GetCellVerticesFromGrid, UpdateParticlePosition, TrilinearInterpolation_Vector) runs on the
 *     host with the reference's operations in the reference's order, so post-processing and other
 *     callers of single cells get the reference's bits (no fused multiply-adds: this file turns
 *     FP contraction off);
 *   - LocateAllParticlesInGrid_TEST and LocateParticleOrFindMigrationTarget_TEST walk every
 *     particle that needs a location on the GPU (fdf_LocatePoints, the reference walk bit for bit);
 *   - InterpolateAllFieldsToSwarm makes the corner field and every particle's velocity on the GPU
 *     (fdf_InterpolatePoints);
 *   - ScatterAllParticleFieldsToEulerFields and CalculateParticleCountPerCell make ParticleCount
 *     and the P average on the GPU (fdf_SetSwarm, fdf_ScatterAllParticleFieldsToEulerFields);
 *   - UpdateAllParticlePositions, ResetAllParticleStatuses and the two CheckAndRemove functions
 *     stay host loops over the DMSwarm fields: one pass over the arrays costs less than moving
 *     them to the GPU and back, and the removals are DMSwarm container operations, done in the
 *     reference's order (backwards, DMSwarmRemovePointAtIndex) so the swarm ends in the same order.
 *
 * One rank holds the whole grid and the whole swarm (the GPU library's model): the walk's
 * migration branch and GuessParticleOwnerWithBBox never change a result, and a DMDA split over
 * several ranks is refused with PETSC_ERR_SUP.  Errors of the library arrive as its PETSc codes
 * (83 for a degenerate face met by the walk, as the reference's CHKERRQ chain).
 *
 * GPU context: each UserCtx is bound to one context on first use (FdfShimAttach makes the
 * binding explicit and picks the device; otherwise the device is $FDF_DEVICE or 0).  The grid
 * is uploaded when the coordinate vector changes and ucat (user->lUcat) when it changes
 * (PetscObjectStateGet), so steps re-send only the swarm arrays they need.
 */
#if defined(__clang__)
#pragma STDC FP_CONTRACT OFF
#elif defined(__GNUC__)
#pragma GCC optimize("fp-contract=off")
#endif

#include "common.h"
#include "walkingsearch.h"
#include "ParticleSwarm.h"
#include "ParticleMotion.h"
#include "interpolation.h"
#include "fdf_gb300.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

_Static_assert(sizeof(PetscReal) == sizeof(double), "the GPU library computes in double precision");

#define SHIM_INTERP_DIST_TOL 1e-14          /* ParticleSwarm.c:5 */

/* ------------------------------------------------------------------ bindings to GPU contexts */

typedef struct {
  UserCtx *user;
  FdfContext *ctx;
  Vec coor_vec;
  PetscObjectState coor_state;
  int has_grid;
  Vec ucat_vec;
  PetscObjectState ucat_state;
  int has_ucat;
} ShimBinding;

#define SHIM_MAX_BINDINGS 16
static ShimBinding g_bind[SHIM_MAX_BINDINGS];

#define FDF_CHECK(b, call)                                                                        \
  do {                                                                                            \
    int e_ = (call);                                                                              \
    if (e_) SETERRQ(PETSC_COMM_SELF, e_, "GPU path: %s", fdf_GetLastError((b)->ctx));             \
  } while (0)

/* Binds user to a GPU context on `device` (an existing binding is kept). */
PetscErrorCode FdfShimAttach(UserCtx *user, int device) {
  if (!user) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "FdfShimAttach: user is NULL");
  ShimBinding *freeb = NULL;
  for (int q = 0; q < SHIM_MAX_BINDINGS; ++q) {
    if (g_bind[q].user == user) return 0;
    if (!g_bind[q].user && !freeb) freeb = &g_bind[q];
  }
  if (!freeb) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "FdfShimAttach: more than %d bound UserCtx", SHIM_MAX_BINDINGS);
  memset(freeb, 0, sizeof *freeb);
  int e = fdf_ContextCreate(&freeb->ctx, device);
  if (e) SETERRQ(PETSC_COMM_SELF, e, "FdfShimAttach: no usable CUDA device %d", device);
  freeb->user = user;
  return 0;
}

/* Releases the GPU context bound to user (no-op when there is none). */
PetscErrorCode FdfShimDetach(UserCtx *user) {
  for (int q = 0; q < SHIM_MAX_BINDINGS; ++q)
    if (user && g_bind[q].user == user) {
      fdf_ContextDestroy(g_bind[q].ctx);
      memset(&g_bind[q], 0, sizeof g_bind[q]);
    }
  return 0;
}

/* The GPU context bound to user, for callers that also use the fdf_* calls directly. */
FdfContext *FdfShimContext(UserCtx *user) {
  for (int q = 0; q < SHIM_MAX_BINDINGS; ++q)
    if (user && g_bind[q].user == user) return g_bind[q].ctx;
  return NULL;
}

static PetscErrorCode binding(UserCtx *user, ShimBinding **out) {
  if (!user) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "UserCtx is NULL");
  for (int pass = 0; pass < 2; ++pass) {
    for (int q = 0; q < SHIM_MAX_BINDINGS; ++q)
      if (g_bind[q].user == user) { *out = &g_bind[q]; return 0; }
    const char *dev = getenv("FDF_DEVICE");
    PetscCall(FdfShimAttach(user, dev ? atoi(dev) : 0));
  }
  SETERRQ(PETSC_COMM_SELF, PETSC_ERR_LIB, "no GPU context for this UserCtx");
}

/* Uploads the node coordinates when the coordinate vector changed (one rank: every node). */
static PetscErrorCode sync_grid(UserCtx *user, ShimBinding *b) {
  Vec coords;
  PetscObjectState st;
  PetscCall(DMGetCoordinatesLocal(user->da, &coords));
  PetscCall(PetscObjectStateGet((PetscObject)coords, &st));
  if (b->has_grid && coords == b->coor_vec && st == b->coor_state) return 0;
  PetscInt n;
  PetscCall(VecGetLocalSize(coords, &n));
  const PetscInt nn = (user->IM + 1) * (user->JM + 1) * (user->KM + 1);
  if (n != 3 * nn)
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "the GPU path needs the whole grid on one rank (%lld of %lld coordinates)",
            (long long)n, (long long)(3 * nn));
  const PetscScalar *c;
  PetscCall(VecGetArrayRead(coords, &c));
  const int e = fdf_SetGrid(b->ctx, user->IM, user->JM, user->KM, c);
  PetscCall(VecRestoreArrayRead(coords, &c));
  FDF_CHECK(b, e);
  b->coor_vec = coords;
  b->coor_state = st;
  b->has_grid = 1;
  b->has_ucat = 0;   /* a new grid drops the context's fields */
  return 0;
}

/* Uploads the cell-centred Cartesian velocity (user->lUcat, node-sized) when it changed. */
static PetscErrorCode sync_ucat(UserCtx *user, ShimBinding *b) {
  PetscObjectState st;
  if (!user->lUcat) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "user->lUcat is NULL");
  PetscCall(PetscObjectStateGet((PetscObject)user->lUcat, &st));
  if (b->has_ucat && user->lUcat == b->ucat_vec && st == b->ucat_state) return 0;
  PetscInt n;
  PetscCall(VecGetLocalSize(user->lUcat, &n));
  if (n != 3 * (user->IM + 1) * (user->JM + 1) * (user->KM + 1))
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "the GPU path needs the whole ucat field on one rank");
  const PetscScalar *u;
  PetscCall(VecGetArrayRead(user->lUcat, &u));
  const int e = fdf_SetUcat(b->ctx, u, 1);
  PetscCall(VecRestoreArrayRead(user->lUcat, &u));
  FDF_CHECK(b, e);
  b->ucat_vec = user->lUcat;
  b->ucat_state = st;
  b->has_ucat = 1;
  return 0;
}

/* ------------------------------------------------------- per-cell arithmetic (host, exact) */

/* walkingsearch.c:25-59: the mean length of the cell's 12 edges. */
PetscErrorCode GetCellCharacteristicSize(const Cell *cell, PetscReal *cellSize) {
  static const int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                  {6, 7}, {7, 4}, {0, 7}, {1, 6}, {2, 5}, {3, 4}};
  if (!cell || !cellSize) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "GetCellCharacteristicSize: Null pointer(s).");
  PetscReal total = 0.0;
  for (int e = 0; e < 12; ++e) {
    const Cmpnts a = cell->vertices[edge[e][0]], b = cell->vertices[edge[e][1]];
    const PetscReal dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    total += sqrt(dx * dx + dy * dy + dz * dz);
  }
  *cellSize = total / 12.0;
  return 0;
}

/* walkingsearch.c:102-227: distance from p to the plane of face (v1, v2, v3, v4), positive on the
 * side of the cell centroid; |d| below the threshold is zero. */
PetscErrorCode ComputeSignedDistanceToPlane(const Cmpnts v1, const Cmpnts v2, const Cmpnts v3, const Cmpnts v4,
                                            const Cmpnts cell_centroid, const Cmpnts p_target, PetscReal *d_signed,
                                            const PetscReal threshold) {
  if (!d_signed) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "Output pointer 'd_signed' is NULL.");
  const PetscReal ax = v2.x - v1.x, ay = v2.y - v1.y, az = v2.z - v1.z;
  const PetscReal bx = v4.x - v1.x, by = v4.y - v1.y, bz = v4.z - v1.z;
  PetscReal nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
  const PetscReal mag = sqrt(nx * nx + ny * ny + nz * nz);
  if (mag < 1.0e-12)
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_USER, "Degenerate plane detected (normal vector is near zero).");
  const PetscReal fx = 0.25 * (v1.x + v2.x + v3.x + v4.x);
  const PetscReal fy = 0.25 * (v1.y + v2.y + v3.y + v4.y);
  const PetscReal fz = 0.25 * (v1.z + v2.z + v3.z + v4.z);
  const PetscReal toward = nx * (cell_centroid.x - fx) + ny * (cell_centroid.y - fy) + nz * (cell_centroid.z - fz);
  if (toward > 1.0e-9) { nx = -nx; ny = -ny; nz = -nz; }   /* normal away from the centroid */
  nx /= mag; ny /= mag; nz /= mag;
  PetscReal d = (fx - p_target.x) * nx + (fy - p_target.y) * ny + (fz - p_target.z) * nz;
  if (fabs(d) < threshold) d = 0.0;
  *d_signed = d;
  return 0;
}

/* walkingsearch.c:271-389: the six faces, each as (v1, v2, v3, v4) of the walk's vertex order. */
PetscErrorCode CalculateDistancesToCellFaces(const Cmpnts p, const Cell *cell, PetscReal *d, const PetscReal threshold) {
  static const int face[6][5] = {{BACK, 0, 3, 2, 1}, {FRONT, 4, 7, 6, 5}, {BOTTOM, 0, 1, 6, 7},
                                 {TOP, 3, 4, 5, 2},  {LEFT, 0, 7, 4, 3},  {RIGHT, 1, 2, 5, 6}};
  if (!cell || !d) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "CalculateDistancesToCellFaces: Null pointer(s).");
  Cmpnts cc = {0.0, 0.0, 0.0};
  for (int v = 0; v < 8; ++v) { cc.x += cell->vertices[v].x; cc.y += cell->vertices[v].y; cc.z += cell->vertices[v].z; }
  cc.x /= 8.0; cc.y /= 8.0; cc.z /= 8.0;
  const Cmpnts *v = cell->vertices;
  for (int f = 0; f < 6; ++f)
    PetscCall(ComputeSignedDistanceToPlane(v[face[f][1]], v[face[f][2]], v[face[f][3]], v[face[f][4]], cc, p,
                                           &d[face[f][0]], threshold));
  return 0;
}

/* walkingsearch.c:407-462: 0 inside; 1, 2 or 3 on that many faces (>= 3 gives 3), accepted even
 * when another face says outside; -1 outside. */
PetscErrorCode DeterminePointPosition(PetscReal *d, PetscInt *result) {
  if (!d || !result) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "DeterminePointPosition: Null pointer(s).");
  int inside = 1;
  PetscInt zeros = 0;
  for (int f = 0; f < NUM_FACES; ++f) {
    if (d[f] < 0.0) inside = 0;
    if (d[f] == 0.0) zeros++;
  }
  *result = inside ? 0 : (zeros == 0 ? -1 : (zeros > 3 ? 3 : zeros));
  return 0;
}

/* walkingsearch.c:521-549: vertices 0..7 = (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k) (i,j+1,k+1)
 * (i+1,j+1,k+1) (i+1,j,k+1) (i,j,k+1) of a [k][j][i] node array. */
PetscErrorCode GetCellVerticesFromGrid(Cmpnts ***coor, PetscInt idx, PetscInt idy, PetscInt idz, Cell *cell) {
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}};
  if (!coor || !cell) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "GetCellVerticesFromGrid: Null pointer(s).");
  for (int v = 0; v < 8; ++v) cell->vertices[v] = coor[idz + off[v][2]][idy + off[v][1]][idx + off[v][0]];
  return 0;
}

/* walkingsearch.c:811-859: the threshold scales with the cell size, then the faces classify p. */
PetscErrorCode EvaluateParticlePosition(const Cell *cell, PetscReal *d, const Cmpnts p, PetscInt *position,
                                        const PetscReal threshold) {
  if (!cell || !d || !position) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "EvaluateParticlePosition: Null pointer(s).");
  PetscReal size;
  PetscCall(GetCellCharacteristicSize(cell, &size));
  PetscCall(CalculateDistancesToCellFaces(p, cell, d, threshold * size));
  return DeterminePointPosition(d, position);
}

/* walkingsearch.c:882-959: one step toward the point; k, then i, then j, the lower face first
 * in i and j, FRONT first in k; no clamping. */
PetscErrorCode UpdateCellIndicesBasedOnDistancesTEST(PetscReal d[NUM_FACES], PetscInt *idx, PetscInt *idy,
                                                     PetscInt *idz) {
  if (!d || !idx || !idy || !idz) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "Null pointer(s).");
  if (d[FRONT] < 0.0) ++*idz; else if (d[BACK] < 0.0) --*idz;
  if (d[LEFT] < 0.0) --*idx; else if (d[RIGHT] < 0.0) ++*idx;
  if (d[BOTTOM] < 0.0) --*idy; else if (d[TOP] < 0.0) ++*idy;
  return 0;
}

/* ParticleSwarm.c:1010-1047: every distance at or below 1e-14 becomes 1e-14 (in d itself), then
 * the three ratios; the k weight is BACK over FRONT + BACK. */
PetscErrorCode UpdateParticleWeights(PetscReal *d, Particle *particle) {
  if (!d || !particle) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "UpdateParticleWeights: Null pointer(s).");
  for (int f = 0; f < NUM_FACES; ++f)
    if (d[f] <= SHIM_INTERP_DIST_TOL) d[f] = SHIM_INTERP_DIST_TOL;
  particle->weights.x = d[LEFT] / (d[LEFT] + d[RIGHT]);
  particle->weights.y = d[BOTTOM] / (d[BOTTOM] + d[TOP]);
  particle->weights.z = d[BACK] / (d[FRONT] + d[BACK]);
  return 0;
}

/* ParticleMotion.c:19-29: explicit Euler with user->dt. */
PetscErrorCode UpdateParticlePosition(UserCtx *user, Cmpnts *position, const Cmpnts *velocity) {
  position->x += velocity->x * user->dt;
  position->y += velocity->y * user->dt;
  position->z += velocity->z * user->dt;
  return 0;
}

/* interpolation.c:839-864 and :957-1042: weights of the 8 corners (0,0,0) .. (1,1,1) from the
 * clamped (a1, a2, a3), accumulated in that order, then divided by their sum. */
PetscErrorCode TrilinearInterpolation_Vector(const char *fieldName, Cmpnts ***fieldVec, PetscInt i, PetscInt j,
                                             PetscInt k, PetscReal a1, PetscReal a2, PetscReal a3, Cmpnts *vec) {
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  (void)fieldName;
  a1 = PetscMax(0.0, PetscMin(1.0, a1));
  a2 = PetscMax(0.0, PetscMin(1.0, a2));
  a3 = PetscMax(0.0, PetscMin(1.0, a3));
  const PetscReal b1 = 1.0 - a1, b2 = 1.0 - a2, b3 = 1.0 - a3;
  const PetscReal w[8] = {b1 * b2 * b3, a1 * b2 * b3, b1 * a2 * b3, a1 * a2 * b3,
                          b1 * b2 * a3, a1 * b2 * a3, b1 * a2 * a3, a1 * a2 * a3};
  PetscReal sum = 0.0, x = 0.0, y = 0.0, z = 0.0;
  for (int c = 0; c < 8; ++c) {
    const Cmpnts q = fieldVec[k + off[c][2]][j + off[c][1]][i + off[c][0]];
    x += w[c] * q.x;
    y += w[c] * q.y;
    z += w[c] * q.z;
    sum += w[c];
  }
  if (sum > 1.0e-14) { vec->x = x / sum; vec->y = y / sum; vec->z = z / sum; }
  else { vec->x = 0.0; vec->y = 0.0; vec->z = 0.0; }
  return 0;
}

/* ------------------------------------------------------------- swarm helpers */

typedef struct {
  DM sw;
  PetscInt n;
  PetscReal *pos, *vel, *wgt, *P;
  PetscInt *cell, *status;
  PetscInt64 *pid;
} Fields;

static const char *const FIELD_NAMES[7] = {"position", "velocity", "weight", "P", "DMSwarm_CellID",
                                           "DMSwarm_location_status", "DMSwarm_pid"};

/* Gets the fields named by mask bits (1 position, 2 velocity, 4 weight, 8 P, 16 CellID,
 * 32 status, 64 pid); release with put_fields and the same mask. */
static PetscErrorCode get_fields(DM sw, unsigned mask, Fields *f) {
  memset(f, 0, sizeof *f);
  f->sw = sw;
  PetscCall(DMSwarmGetLocalSize(sw, &f->n));
  void **slot[7] = {(void **)&f->pos, (void **)&f->vel, (void **)&f->wgt, (void **)&f->P,
                    (void **)&f->cell, (void **)&f->status, (void **)&f->pid};
  for (int q = 0; q < 7; ++q)
    if (mask & (1u << q)) PetscCall(DMSwarmGetField(sw, FIELD_NAMES[q], NULL, NULL, slot[q]));
  return 0;
}
static PetscErrorCode put_fields(Fields *f, unsigned mask) {
  void **slot[7] = {(void **)&f->pos, (void **)&f->vel, (void **)&f->wgt, (void **)&f->P,
                    (void **)&f->cell, (void **)&f->status, (void **)&f->pid};
  for (int q = 0; q < 7; ++q)
    if ((mask & (1u << q)) && *slot[q]) PetscCall(DMSwarmRestoreField(f->sw, FIELD_NAMES[q], NULL, NULL, slot[q]));
  return 0;
}

/* ---------------------------------------------------------- swarm-level functions */

/* ParticleMotion.c:2149-2176: ACTIVE_AND_LOCATED -> NEEDS_LOCATION; other statuses stay. */
PetscErrorCode ResetAllParticleStatuses(UserCtx *user) {
  Fields f;
  PetscCall(get_fields(user->swarm, 32u, &f));
  for (PetscInt p = 0; p < f.n; ++p)
    if (f.status[p] == ACTIVE_AND_LOCATED) f.status[p] = NEEDS_LOCATION;
  return put_fields(&f, 32u);
}

/* ParticleMotion.c:38-95: position += velocity * dt for every particle. */
PetscErrorCode UpdateAllParticlePositions(UserCtx *user) {
  Fields f;
  PetscCall(get_fields(user->swarm, 3u, &f));
  for (PetscInt p = 0; p < f.n; ++p) {
    Cmpnts x = {f.pos[3 * p], f.pos[3 * p + 1], f.pos[3 * p + 2]};
    const Cmpnts v = {f.vel[3 * p], f.vel[3 * p + 1], f.vel[3 * p + 2]};
    UpdateParticlePosition(user, &x, &v);
    f.pos[3 * p] = x.x; f.pos[3 * p + 1] = x.y; f.pos[3 * p + 2] = x.z;
  }
  return put_fields(&f, 3u);
}

/* The walk of `m` particles (slots `slot`) on the GPU; results written into the fields. */
static PetscErrorCode walk_slots(ShimBinding *b, Fields *f, const PetscInt *slot, PetscInt m) {
  if (m == 0) return 0;
  double *pos = (double *)malloc(24 * (size_t)m), *w = (double *)malloc(24 * (size_t)m);
  int64_t *cin = (int64_t *)malloc(24 * (size_t)m), *cout = (int64_t *)malloc(24 * (size_t)m);
  int64_t *st = (int64_t *)malloc(8 * (size_t)m);
  int e = (pos && w && cin && cout && st) ? 0 : FDF_ERR_MEM;
  if (!e) {
    for (PetscInt t = 0; t < m; ++t)
      for (int c = 0; c < 3; ++c) {
        pos[3 * t + c] = f->pos[3 * slot[t] + c];
        cin[3 * t + c] = (int64_t)f->cell[3 * slot[t] + c];
      }
    e = fdf_LocatePoints(b->ctx, m, pos, cin, cout, w, st);
  }
  if (!e)
    for (PetscInt t = 0; t < m; ++t) {
      const PetscInt q = slot[t];
      for (int c = 0; c < 3; ++c) f->cell[3 * q + c] = (PetscInt)cout[3 * t + c];
      f->status[q] = (PetscInt)st[t];
      if (st[t] == ACTIVE_AND_LOCATED)   /* a LOST particle keeps its weights, as in the reference */
        for (int c = 0; c < 3; ++c) f->wgt[3 * q + c] = w[3 * t + c];
    }
  free(pos); free(w); free(cin); free(cout); free(st);
  if (e == FDF_ERR_MEM) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_MEM, "walk: out of host memory");
  FDF_CHECK(b, e);
  return 0;
}

/* ParticleMotion.c:1931-2135 on one rank: every particle not ACTIVE_AND_LOCATED is walked
 * (from its previous cell, or from the corner cell when it has none), and its cell, status and
 * -- when located -- weights are written back.  bboxlist is not needed: on one rank the box
 * guess can only answer this rank, and both of its branches walk. */
PetscErrorCode LocateAllParticlesInGrid_TEST(UserCtx *user, BoundingBox *bboxlist) {
  (void)bboxlist;
  ShimBinding *b;
  PetscCall(binding(user, &b));
  PetscCall(sync_grid(user, b));
  const unsigned mask = 1u | 4u | 16u | 32u;
  Fields f;
  PetscCall(get_fields(user->swarm, mask, &f));
  PetscInt *slot = (PetscInt *)malloc(sizeof(PetscInt) * (size_t)(f.n > 0 ? f.n : 1));
  PetscErrorCode e = slot ? 0 : PETSC_ERR_MEM;
  PetscInt m = 0;
  if (!e) {
    for (PetscInt p = 0; p < f.n; ++p)
      if (f.status[p] != ACTIVE_AND_LOCATED) slot[m++] = p;
    e = walk_slots(b, &f, slot, m);
  }
  free(slot);
  PetscCall(put_fields(&f, mask));
  return e;
}

/* walkingsearch.c:1094-1242 for one particle: cell, status and (when located) weights. */
PetscErrorCode LocateParticleOrFindMigrationTarget_TEST(UserCtx *user, Particle *particle,
                                                        ParticleLocationStatus *status_out) {
  if (!user || !particle || !status_out)
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "LocateParticleOrFindMigrationTarget_TEST: Null pointer(s).");
  ShimBinding *b;
  PetscCall(binding(user, &b));
  PetscCall(sync_grid(user, b));
  const double pos[3] = {particle->loc.x, particle->loc.y, particle->loc.z};
  const int64_t cin[3] = {particle->cell[0], particle->cell[1], particle->cell[2]};
  int64_t cout[3], st;
  double w[3];
  FDF_CHECK(b, fdf_LocatePoints(b->ctx, 1, pos, cin, cout, w, &st));
  for (int c = 0; c < 3; ++c) particle->cell[c] = (PetscInt)cout[c];
  if (st == ACTIVE_AND_LOCATED) { particle->weights.x = w[0]; particle->weights.y = w[1]; particle->weights.z = w[2]; }
  *status_out = (ParticleLocationStatus)st;
  return 0;
}

/* ParticleMotion.c:532-625 and :283-383: backwards over the swarm, each removal moving the last
 * particle into the freed slot (DMSwarmRemovePointAtIndex), as the reference does. */
static PetscErrorCode remove_where(UserCtx *user, const BoundingBox *bboxlist, PetscInt *local, PetscInt *global) {
  DM sw = user->swarm;
  PetscInt removed = 0;
  if (!local) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "removed-count pointer is NULL");
  *local = 0;
  if (global) *global = 0;
  const unsigned mask = bboxlist ? 1u : 32u;
  Fields f;
  PetscCall(get_fields(sw, mask, &f));
  for (PetscInt p = f.n - 1; p >= 0; --p) {
    int drop;
    if (bboxlist) {
      const BoundingBox *bb = &bboxlist[0];
      const PetscReal x = f.pos[3 * p], y = f.pos[3 * p + 1], z = f.pos[3 * p + 2];
      drop = !(x >= bb->min_coords.x && x <= bb->max_coords.x && y >= bb->min_coords.y && y <= bb->max_coords.y &&
               z >= bb->min_coords.z && z <= bb->max_coords.z);
    } else {
      drop = f.status[p] == LOST;
    }
    if (!drop) continue;
    PetscCall(put_fields(&f, mask));   /* the swarm may not be resized while its fields are held */
    PetscCall(DMSwarmRemovePointAtIndex(sw, p));
    removed++;
    PetscCall(get_fields(sw, mask, &f));
  }
  PetscCall(put_fields(&f, mask));
  *local = removed;
  if (global) *global = removed;
  return 0;
}

PetscErrorCode CheckAndRemoveLostParticles(UserCtx *user, PetscInt *removedCountLocal, PetscInt *removedCountGlobal) {
  return remove_where(user, NULL, removedCountLocal, removedCountGlobal);
}

PetscErrorCode CheckAndRemoveOutOfBoundsParticles(UserCtx *user, PetscInt *removedCountLocal,
                                                  PetscInt *removedCountGlobal, const BoundingBox *bboxlist) {
  if (!bboxlist) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "bboxlist is NULL");
  return remove_where(user, bboxlist, removedCountLocal, removedCountGlobal);
}

/* interpolation.c:1660-1711 (InterpolateEulerFieldToSwarm of user->lUcat into "velocity"):
 * corner field and trilinear interpolation on the GPU, in the swarm's order. */
PetscErrorCode InterpolateAllFieldsToSwarm(UserCtx *user) {
  ShimBinding *b;
  PetscCall(binding(user, &b));
  PetscCall(sync_grid(user, b));
  PetscCall(sync_ucat(user, b));
  const unsigned mask = 2u | 4u | 16u;
  Fields f;
  PetscCall(get_fields(user->swarm, mask, &f));
  int64_t *cell = (int64_t *)malloc(24 * (size_t)(f.n > 0 ? f.n : 1));
  int e = cell ? 0 : FDF_ERR_MEM;
  if (!e) {
    for (PetscInt q = 0; q < 3 * f.n; ++q) cell[q] = (int64_t)f.cell[q];
    e = fdf_InterpolatePoints(b->ctx, f.n, cell, f.wgt, f.vel);
  }
  free(cell);
  PetscCall(put_fields(&f, mask));
  if (e == FDF_ERR_MEM) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_MEM, "interpolation: out of host memory");
  FDF_CHECK(b, e);
  return 0;
}

/* ParticleCount and the P average of the swarm on the GPU, node-sized. */
static PetscErrorCode scatter_gpu(UserCtx *user, ShimBinding *b, double *count, double *avg) {
  const unsigned mask = 1u | 2u | 4u | 8u | 16u | 32u | 64u;
  Fields f;
  PetscCall(get_fields(user->swarm, mask, &f));
  int64_t *cell = (int64_t *)malloc(24 * (size_t)(f.n > 0 ? f.n : 1));
  int64_t *st = (int64_t *)malloc(8 * (size_t)(f.n > 0 ? f.n : 1));
  int e = (cell && st) ? 0 : FDF_ERR_MEM;
  if (!e) {
    for (PetscInt q = 0; q < 3 * f.n; ++q) cell[q] = (int64_t)f.cell[q];
    for (PetscInt q = 0; q < f.n; ++q) st[q] = (int64_t)f.status[q];
    e = fdf_SetSwarm(b->ctx, f.n, f.pos, f.vel, f.wgt, f.P, cell, (const int64_t *)f.pid, st);
  }
  if (!e) e = fdf_ScatterAllParticleFieldsToEulerFields(b->ctx);
  if (!e) e = fdf_GetScatteredFields(b->ctx, count, avg);
  free(cell); free(st);
  PetscCall(put_fields(&f, mask));
  if (e == FDF_ERR_MEM) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_MEM, "scatter: out of host memory");
  FDF_CHECK(b, e);
  return 0;
}

static PetscErrorCode write_node_field(UserCtx *user, Vec v, const double *src) {
  PetscInt n;
  PetscCall(VecGetLocalSize(v, &n));
  if (n != (user->IM + 1) * (user->JM + 1) * (user->KM + 1))
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "the GPU path needs node-sized fields on one rank");
  PetscScalar *a;
  PetscCall(VecGetArray(v, &a));
  memcpy(a, src, sizeof(double) * (size_t)n);
  return VecRestoreArray(v, &a);
}

static PetscErrorCode scatter_into(UserCtx *user, int with_P) {
  ShimBinding *b;
  PetscCall(binding(user, &b));
  PetscCall(sync_grid(user, b));
  const size_t nn = (size_t)((user->IM + 1) * (user->JM + 1) * (user->KM + 1));
  double *count = (double *)malloc(8 * nn), *avg = (double *)malloc(8 * nn);
  PetscErrorCode e = (count && avg) ? scatter_gpu(user, b, count, avg) : PETSC_ERR_MEM;
  if (!e) e = write_node_field(user, user->ParticleCount, count);
  if (!e && with_P) e = write_node_field(user, user->P, avg);
  free(count); free(avg);
  return e;
}

/* ParticleMotion.c:931-1067: particles per cell into user->ParticleCount (node-sized). */
PetscErrorCode CalculateParticleCountPerCell(UserCtx *user) {
  if (!user || !user->ParticleCount)
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "UserCtx or ParticleCount is NULL.");
  return scatter_into(user, 0);
}

/* interpolation.c:2223-2313: ParticleCount, then P summed per cell and divided by the count
 * (0 where the count is 0) into user->P.  The sums run in (cell, PID) order; the reference sums
 * in the swarm's order, which gives the same bits when a cell's P values are equal (the
 * reference's P field is the constant it was initialised with). */
PetscErrorCode ScatterAllParticleFieldsToEulerFields(UserCtx *user) {
  if (!user || !user->ParticleCount)
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE,
            "UserCtx->ParticleCount is NULL. Compute counts before calling ScatterAllParticleFieldsToEulerFields.");
  if (!user->P) return 0;   /* the reference only warns when there is no Eulerian P */
  return scatter_into(user, 1);
}
