/*
 * shim_harness.c -- test entry points that drive fdf_gb300/shim/picurv_shim.c (the reference's
 * function signatures over the GPU library) the way PICurv's host code does: a one-rank UserCtx
 * with its DMDAs, coordinates, ucat, ParticleCount and P vectors, bounding box and cell map, a
 * DMSwarm with the reference's particle fields, and the step's calls in simulation.c's order.
 * Compiled by tests/shim_util.py against tests/petsc_stub (PETSc stand-in) and either the
 * reference's own headers or the stand-ins in tests/petsc_stub/picurv.  Test infrastructure.
 */
#include "common.h"
#include "walkingsearch.h"
#include "ParticleSwarm.h"
#include "ParticleMotion.h"
#include "interpolation.h"

#include <stdint.h>

#define API __attribute__((visibility("default")))

PetscErrorCode FdfShimAttach(UserCtx *user, int device);
PetscErrorCode FdfShimDetach(UserCtx *user);

API const char *shim_last_error(void) { return minipetsc_last_error(); }
API void shim_clear_error(void) { minipetsc_clear_error(); }

/* ---- per-cell functions with array arguments (for ctypes) ---- */
static Cmpnts cm(const double *v) { Cmpnts c; c.x = v[0]; c.y = v[1]; c.z = v[2]; return c; }
static void cell_of(const double *verts, Cell *c) { for (int q = 0; q < 8; ++q) c->vertices[q] = cm(verts + 3 * q); }

API int shim_signed_distance(const double *v1, const double *v2, const double *v3, const double *v4, const double *cc,
                             const double *p, double thr, double *d) {
  return ComputeSignedDistanceToPlane(cm(v1), cm(v2), cm(v3), cm(v4), cm(cc), cm(p), d, thr);
}
API int shim_characteristic_size(const double *verts, double *h) {
  Cell c; cell_of(verts, &c);
  return GetCellCharacteristicSize(&c, h);
}
API int shim_evaluate_position(const double *verts, const double *p, double thr, double *d, int64_t *pos) {
  Cell c; cell_of(verts, &c);
  PetscInt r = 0;
  int e = EvaluateParticlePosition(&c, d, cm(p), &r, thr);
  *pos = r;
  return e;
}
API int shim_point_position(double *d, int64_t *r) {
  PetscInt x = 0;
  int e = DeterminePointPosition(d, &x);
  *r = x;
  return e;
}
API int shim_update_indices(double *d, int64_t *ijk) {
  PetscInt i = ijk[0], j = ijk[1], k = ijk[2];
  int e = UpdateCellIndicesBasedOnDistancesTEST(d, &i, &j, &k);
  ijk[0] = i; ijk[1] = j; ijk[2] = k;
  return e;
}
API int shim_update_weights(double *d, double *w) {
  Particle p;
  memset(&p, 0, sizeof p);
  int e = UpdateParticleWeights(d, &p);
  w[0] = p.weights.x; w[1] = p.weights.y; w[2] = p.weights.z;
  return e;
}

/* ---- one rank of PICurv ---- */
typedef struct {
  UserCtx user;
  BoundingBox bboxlist[1];
  RankCellInfo map[1];
  Vec coords;
} Sim;

static PetscErrorCode fill(Vec v, const double *src, PetscInt n) {
  if (minipetsc_vec_length(v) != n) return PETSC_ERR_ARG_SIZ;
  memcpy(minipetsc_vec_data(v), src, (size_t)n * sizeof(double));
  minipetsc_vec_touch(v);
  return 0;
}

API void *shim_sim_create(int64_t IM, int64_t JM, int64_t KM, const double *coor, const double *ucat, double dt,
                          int device) {
  Sim *s = (Sim *)calloc(1, sizeof(Sim));
  if (!s) return NULL;
  UserCtx *u = &s->user;
  const PetscInt M = IM + 1, N = JM + 1, P = KM + 1, Nn = M * N * P;
  u->IM = IM; u->JM = JM; u->KM = KM;
  u->dt = dt;
  if (minipetsc_dmda_create(M, N, P, 1, &u->da) || minipetsc_dmda_create(M, N, P, 3, &u->fda) ||
      minipetsc_vec_create(u->fda, 3 * Nn, 3, &s->coords) || fill(s->coords, coor, 3 * Nn) ||
      minipetsc_dm_set_coordinates(u->da, u->fda, s->coords) || minipetsc_dm_set_coordinates(u->fda, u->fda, s->coords) ||
      DMDAGetLocalInfo(u->da, &u->info) || DMCreateGlobalVector(u->fda, &u->Ucat) ||
      DMCreateLocalVector(u->fda, &u->lUcat) || DMCreateGlobalVector(u->da, &u->P) ||
      DMCreateGlobalVector(u->da, &u->ParticleCount)) {
    free(s);
    return NULL;
  }
  if (ucat && (fill(u->Ucat, ucat, 3 * Nn) || fill(u->lUcat, ucat, 3 * Nn))) { free(s); return NULL; }
  u->neighbors.rank_xm = u->neighbors.rank_xp = u->neighbors.rank_ym = MPI_PROC_NULL;
  u->neighbors.rank_yp = u->neighbors.rank_zm = u->neighbors.rank_zp = MPI_PROC_NULL;
  s->map[0].xs_cell = 0; s->map[0].ys_cell = 0; s->map[0].zs_cell = 0;
  s->map[0].xm_cell = IM; s->map[0].ym_cell = JM; s->map[0].zm_cell = KM;
  u->RankCellInfoMap = s->map;
  /* the rank's box: node extremes widened by 1e-6 (grid.c:816-858) */
  double lo[3] = {PETSC_MAX_REAL, PETSC_MAX_REAL, PETSC_MAX_REAL}, hi[3] = {PETSC_MIN_REAL, PETSC_MIN_REAL, PETSC_MIN_REAL};
  for (PetscInt q = 0; q < Nn; ++q)
    for (int c = 0; c < 3; ++c) {
      if (coor[3 * q + c] < lo[c]) lo[c] = coor[3 * q + c];
      if (coor[3 * q + c] > hi[c]) hi[c] = coor[3 * q + c];
    }
  u->bbox.min_coords.x = lo[0] - 1e-6; u->bbox.min_coords.y = lo[1] - 1e-6; u->bbox.min_coords.z = lo[2] - 1e-6;
  u->bbox.max_coords.x = hi[0] + 1e-6; u->bbox.max_coords.y = hi[1] + 1e-6; u->bbox.max_coords.z = hi[2] + 1e-6;
  s->bboxlist[0] = u->bbox;
  /* the swarm with the reference's fields (ParticleSwarm.c:64-96) */
  if (DMCreate(PETSC_COMM_WORLD, &u->swarm) || DMSetType(u->swarm, DMSWARM) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "position", 3, PETSC_REAL) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "velocity", 3, PETSC_REAL) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "DMSwarm_CellID", 3, PETSC_INT) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "weight", 3, PETSC_REAL) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "P", 1, PETSC_REAL) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "pos_phy", 3, PETSC_REAL) ||
      DMSwarmRegisterPetscDatatypeField(u->swarm, "DMSwarm_location_status", 1, PETSC_INT) ||
      DMSwarmFinalizeFieldRegister(u->swarm) || DMSwarmSetLocalSizes(u->swarm, 0, 0)) {
    free(s);
    return NULL;
  }
  if (device >= 0 && FdfShimAttach(u, device)) { free(s); return NULL; }
  return s;
}

API void *shim_sim_user(void *h) { return &((Sim *)h)->user; }

API void shim_sim_destroy(void *h) {
  Sim *s = (Sim *)h;
  if (!s) return;
  UserCtx *u = &s->user;
  FdfShimDetach(u);
  VecDestroy(&u->Ucat); VecDestroy(&u->lUcat); VecDestroy(&u->P); VecDestroy(&u->ParticleCount);
  VecDestroy(&s->coords);
  DMDestroy(&u->swarm); DMDestroy(&u->da); DMDestroy(&u->fda);
  free(s);
}

API int shim_set_ucat(void *h, const double *ucat) {
  Sim *s = (Sim *)h;
  const PetscInt n = minipetsc_vec_length(s->user.lUcat);
  PetscCall(fill(s->user.Ucat, ucat, n));
  return fill(s->user.lUcat, ucat, n);
}

API int shim_swarm_set(void *h, int64_t n, const double *pos, const double *vel, const double *wgt, const double *P,
                       const int64_t *cell, const int64_t *pid, const int64_t *status) {
  DM sw = ((Sim *)h)->user.swarm;
  PetscCall(DMSwarmSetLocalSizes(sw, n, 0));
  double *fp; PetscInt *fi; PetscInt64 *fl;
  PetscCall(DMSwarmGetField(sw, "position", NULL, NULL, (void **)&fp)); memcpy(fp, pos, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "position", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "velocity", NULL, NULL, (void **)&fp)); memcpy(fp, vel, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "velocity", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "weight", NULL, NULL, (void **)&fp)); memcpy(fp, wgt, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "weight", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "P", NULL, NULL, (void **)&fp)); memcpy(fp, P, 8 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "P", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  for (int64_t q = 0; q < 3 * n; ++q) fi[q] = cell[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  for (int64_t q = 0; q < n; ++q) fi[q] = status[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  for (int64_t q = 0; q < n; ++q) fl[q] = pid[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  return 0;
}

API int shim_swarm_size(void *h, int64_t *n) {
  PetscInt m;
  PetscCall(DMSwarmGetLocalSize(((Sim *)h)->user.swarm, &m));
  *n = m;
  return 0;
}

API int shim_swarm_get(void *h, double *pos, double *vel, double *wgt, double *P, int64_t *cell, int64_t *pid,
                       int64_t *status) {
  DM sw = ((Sim *)h)->user.swarm;
  PetscInt n;
  PetscCall(DMSwarmGetLocalSize(sw, &n));
  double *fp; PetscInt *fi; PetscInt64 *fl;
  PetscCall(DMSwarmGetField(sw, "position", NULL, NULL, (void **)&fp)); memcpy(pos, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "position", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "velocity", NULL, NULL, (void **)&fp)); memcpy(vel, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "velocity", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "weight", NULL, NULL, (void **)&fp)); memcpy(wgt, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "weight", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "P", NULL, NULL, (void **)&fp)); memcpy(P, fp, 8 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "P", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  for (PetscInt q = 0; q < 3 * n; ++q) cell[q] = fi[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  for (PetscInt q = 0; q < n; ++q) status[q] = fi[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(sw, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  for (PetscInt q = 0; q < n; ++q) pid[q] = fl[q];
  PetscCall(DMSwarmRestoreField(sw, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  return 0;
}

/* The step's calls one by one (simulation.c:248-292): 0 ResetAllParticleStatuses,
 * 1 UpdateAllParticlePositions, 2 LocateAllParticlesInGrid_TEST, 3 CheckAndRemoveLostParticles,
 * 4 CheckAndRemoveOutOfBoundsParticles, 5 InterpolateAllFieldsToSwarm,
 * 6 ScatterAllParticleFieldsToEulerFields, 7 CalculateParticleCountPerCell. */
API int shim_stage(void *h, int stage, int64_t *removed) {
  Sim *s = (Sim *)h;
  UserCtx *u = &s->user;
  PetscInt loc = 0, glob = 0;
  int e;
  switch (stage) {
    case 0: e = ResetAllParticleStatuses(u); break;
    case 1: e = UpdateAllParticlePositions(u); break;
    case 2: e = LocateAllParticlesInGrid_TEST(u, s->bboxlist); break;
    case 3: e = CheckAndRemoveLostParticles(u, &loc, &glob); break;
    case 4: e = CheckAndRemoveOutOfBoundsParticles(u, &loc, &glob, s->bboxlist); break;
    case 5: e = InterpolateAllFieldsToSwarm(u); break;
    case 6: e = ScatterAllParticleFieldsToEulerFields(u); break;
    case 7: e = CalculateParticleCountPerCell(u); break;
    default: return PETSC_ERR_ARG_OUTOFRANGE;
  }
  if (removed) *removed = loc;
  if (!e && minipetsc_swarm_fields_held(u->swarm))
    return minipetsc_seterr(__func__, __FILE__, __LINE__, PETSC_ERR_ARG_WRONGSTATE, "a swarm field was left held");
  return e;
}

/* LocateParticleOrFindMigrationTarget_TEST for one point through the shim. */
API int shim_locate_point(void *h, const double *p, const int64_t *cell_in, const double *w_in, int64_t *cell_out,
                          double *w, int64_t *status) {
  Particle q;
  memset(&q, 0, sizeof q);
  q.loc = cm(p);
  q.cell[0] = cell_in[0]; q.cell[1] = cell_in[1]; q.cell[2] = cell_in[2];
  q.weights = cm(w_in);
  ParticleLocationStatus st = NEEDS_LOCATION;
  int e = LocateParticleOrFindMigrationTarget_TEST(&((Sim *)h)->user, &q, &st);
  cell_out[0] = q.cell[0]; cell_out[1] = q.cell[1]; cell_out[2] = q.cell[2];
  w[0] = q.weights.x; w[1] = q.weights.y; w[2] = q.weights.z;
  *status = (int64_t)st;
  return e;
}

API int shim_get_scattered(void *h, double *count, double *P) {
  Sim *s = (Sim *)h;
  const PetscInt n = minipetsc_vec_length(s->user.P);
  memcpy(count, minipetsc_vec_data(s->user.ParticleCount), (size_t)n * sizeof(double));
  memcpy(P, minipetsc_vec_data(s->user.P), (size_t)n * sizeof(double));
  return 0;
}
