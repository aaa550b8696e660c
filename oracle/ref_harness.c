/*
 * ref_harness.c -- entry points into the reference's own particle-path code, compiled from the
 * unmodified sources (walkingsearch.c, ParticleSwarm.c, interpolation.c, ParticleMotion.c,
 * grid.c) against the one-rank PETSc stand-in in tests/petsc_stub.  Test infrastructure: the
 * recipe oracle/ref_build.py builds oracle/_ref/libpicurv_ref.so from these, and the tests use
 * it to pin the CPU restatement (picurv_oracle.c) and to write golden vectors.
 *
 * The harness only builds the objects a one-rank run of the reference holds (UserCtx with its
 * DMDAs, coordinates, ucat, ParticleCount and P vectors, bounding box, cell-ownership map, and
 * a DMSwarm with the reference's own fields from RegisterParticleFields) and calls the
 * reference's functions in the order simulation.c does (simulation.c:129-175, 240-297).
 * The reference's logging (logging.c) is not part of the path; quiet stand-ins for its
 * level and allow-list queries keep every LOG_ALLOW silent.
 */
#include "common.h"
#include "logging.h"
#include "walkingsearch.h"
#include "ParticleSwarm.h"
#include "ParticleMotion.h"
#include "interpolation.h"
#include "grid.h"

#define REF_API __attribute__((visibility("default")))

/* ---- logging.c stand-ins (quiet) ---- */
PetscLogEvent EVENT_Individualwalkingsearch = 0, EVENT_walkingsearch = 0, EVENT_GlobalParticleLocation = 0,
              EVENT_IndividualLocation = 0;
LogLevel get_log_level() { return LOG_ERROR; }
PetscBool is_function_allowed(const char *functionName) { (void)functionName; return PETSC_FALSE; }
PetscErrorCode LOG_CELL_VERTICES(const Cell *cell, PetscMPIInt rank) { (void)cell; (void)rank; return 0; }
PetscErrorCode LOG_FACE_DISTANCES(PetscReal *d) { (void)d; return 0; }

REF_API const char *ref_last_error(void) { return minipetsc_last_error(); }
REF_API void ref_clear_error(void) { minipetsc_clear_error(); }
REF_API int ref_petscint_bytes(void) { return (int)sizeof(PetscInt); }

/* ---- per-cell and per-particle functions (walkingsearch.c, ParticleSwarm.c) ---- */
static Cmpnts cm(const double *v) { Cmpnts c; c.x = v[0]; c.y = v[1]; c.z = v[2]; return c; }
static void cell_of(const double *verts, Cell *c) {
  for (int q = 0; q < 8; ++q) c->vertices[q] = cm(verts + 3 * q);
}

REF_API int ref_ComputeSignedDistanceToPlane(const double *v1, const double *v2, const double *v3, const double *v4,
                                             const double *cc, const double *p, double thr, double *d) {
  return ComputeSignedDistanceToPlane(cm(v1), cm(v2), cm(v3), cm(v4), cm(cc), cm(p), d, thr);
}
REF_API int ref_GetCellCharacteristicSize(const double *verts, double *h) {
  Cell c;
  cell_of(verts, &c);
  return GetCellCharacteristicSize(&c, h);
}
REF_API int ref_CalculateDistancesToCellFaces(const double *verts, const double *p, double thr, double *d) {
  Cell c;
  cell_of(verts, &c);
  return CalculateDistancesToCellFaces(cm(p), &c, d, thr);
}
REF_API int ref_DeterminePointPosition(double *d, int64_t *result) {
  PetscInt r = 0;
  int e = DeterminePointPosition(d, &r);
  *result = r;
  return e;
}
REF_API int ref_EvaluateParticlePosition(const double *verts, const double *p, double thr, double *d,
                                         int64_t *position) {
  Cell c;
  cell_of(verts, &c);
  PetscInt r = 0;
  int e = EvaluateParticlePosition(&c, d, cm(p), &r, thr);
  *position = r;
  return e;
}
REF_API int ref_UpdateCellIndicesBasedOnDistancesTEST(double *d, int64_t *ijk) {
  PetscInt i = ijk[0], j = ijk[1], k = ijk[2];
  int e = UpdateCellIndicesBasedOnDistancesTEST(d, &i, &j, &k);
  ijk[0] = i; ijk[1] = j; ijk[2] = k;
  return e;
}
REF_API int ref_UpdateParticleWeights(double *d, double *w) {
  Particle p;
  memset(&p, 0, sizeof p);
  int e = UpdateParticleWeights(d, &p);
  w[0] = p.weights.x; w[1] = p.weights.y; w[2] = p.weights.z;
  return e;
}

/* ---- one rank of the reference: grid, fields, swarm ---- */
typedef struct {
  UserCtx user;
  BoundingBox bboxlist[1];
  RankCellInfo map[1];
  Vec coords;
} RefSim;

static PetscErrorCode fill(Vec v, const double *src, PetscInt n) {
  if (minipetsc_vec_length(v) != n) return PETSC_ERR_ARG_SIZ;
  memcpy(minipetsc_vec_data(v), src, (size_t)n * sizeof(double));
  minipetsc_vec_touch(v);
  return 0;
}

/* coor: node coordinates [KM+1][JM+1][IM+1][3]; ucat (optional): the reference's node-sized
 * cell-centred Cartesian velocity [KM+1][JM+1][IM+1][3]. */
REF_API void *ref_sim_create(int64_t IM, int64_t JM, int64_t KM, const double *coor, const double *ucat, double dt) {
  RefSim *s = (RefSim *)calloc(1, sizeof(RefSim));
  if (!s) return NULL;
  UserCtx *u = &s->user;
  const PetscInt M = IM + 1, N = JM + 1, P = KM + 1, Nn = M * N * P;
  u->IM = IM; u->JM = JM; u->KM = KM;
  u->dt = dt;
  if (minipetsc_dmda_create(M, N, P, 1, &u->da) || minipetsc_dmda_create(M, N, P, 3, &u->fda) ||
      minipetsc_vec_create(u->fda, 3 * Nn, 3, &s->coords) || fill(s->coords, coor, 3 * Nn) ||
      minipetsc_dm_set_coordinates(u->da, u->fda, s->coords) ||
      minipetsc_dm_set_coordinates(u->fda, u->fda, s->coords) || DMDAGetLocalInfo(u->da, &u->info) ||
      DMCreateGlobalVector(u->fda, &u->Ucat) || DMCreateLocalVector(u->fda, &u->lUcat) ||
      DMCreateGlobalVector(u->da, &u->P) || DMCreateGlobalVector(u->da, &u->ParticleCount)) {
    free(s);
    return NULL;
  }
  if (ucat && (fill(u->Ucat, ucat, 3 * Nn) || fill(u->lUcat, ucat, 3 * Nn))) { free(s); return NULL; }
  /* one rank owns every cell and every neighbour is absent (setup.c:679-812) */
  u->neighbors.rank_xm = u->neighbors.rank_xp = MPI_PROC_NULL;
  u->neighbors.rank_ym = u->neighbors.rank_yp = MPI_PROC_NULL;
  u->neighbors.rank_zm = u->neighbors.rank_zp = MPI_PROC_NULL;
  s->map[0].xs_cell = 0; s->map[0].ys_cell = 0; s->map[0].zs_cell = 0;
  s->map[0].xm_cell = IM; s->map[0].ym_cell = JM; s->map[0].zm_cell = KM;
  u->RankCellInfoMap = s->map;
  /* the rank's bounding box, computed by the reference (grid.c) */
  if (ComputeLocalBoundingBox(u, &u->bbox)) { free(s); return NULL; }
  s->bboxlist[0] = u->bbox;
  return s;
}

REF_API int ref_sim_bbox(void *h, double *bb) {
  RefSim *s = (RefSim *)h;
  bb[0] = s->user.bbox.min_coords.x; bb[1] = s->user.bbox.min_coords.y; bb[2] = s->user.bbox.min_coords.z;
  bb[3] = s->user.bbox.max_coords.x; bb[4] = s->user.bbox.max_coords.y; bb[5] = s->user.bbox.max_coords.z;
  return 0;
}

REF_API int ref_sim_set_ucat(void *h, const double *ucat) {
  RefSim *s = (RefSim *)h;
  const PetscInt Nn = (s->user.IM + 1) * (s->user.JM + 1) * (s->user.KM + 1);
  PetscCall(fill(s->user.Ucat, ucat, 3 * Nn));
  return fill(s->user.lUcat, ucat, 3 * Nn);
}

REF_API void ref_sim_destroy(void *h) {
  RefSim *s = (RefSim *)h;
  if (!s) return;
  UserCtx *u = &s->user;
  VecDestroy(&u->Ucat); VecDestroy(&u->lUcat); VecDestroy(&u->P); VecDestroy(&u->ParticleCount);
  VecDestroy(&s->coords);
  DMDestroy(&u->swarm); DMDestroy(&u->da); DMDestroy(&u->fda);
  free(s);
}

/* LocateParticleOrFindMigrationTarget_TEST (walkingsearch.c:1094-1242) for one point. */
REF_API int ref_locate_point(void *h, const double *p, const int64_t *cell_in, int64_t *cell_out, double *w,
                             int64_t *status) {
  RefSim *s = (RefSim *)h;
  Particle q;
  memset(&q, 0, sizeof q);
  q.loc = cm(p);
  q.cell[0] = cell_in[0]; q.cell[1] = cell_in[1]; q.cell[2] = cell_in[2];
  q.location_status = NEEDS_LOCATION;
  ParticleLocationStatus st = NEEDS_LOCATION;
  int e = LocateParticleOrFindMigrationTarget_TEST(&s->user, &q, &st);
  cell_out[0] = q.cell[0]; cell_out[1] = q.cell[1]; cell_out[2] = q.cell[2];
  w[0] = q.weights.x; w[1] = q.weights.y; w[2] = q.weights.z;
  *status = (int64_t)st;
  return e;
}

/* A DMSwarm with the reference's fields (RegisterParticleFields, ParticleSwarm.c:64-96)
 * holding n particles in the given order. */
REF_API int ref_swarm_set(void *h, int64_t n, const double *pos, const double *vel, const double *wgt,
                          const double *P, const int64_t *cell, const int64_t *pid, const int64_t *status) {
  RefSim *s = (RefSim *)h;
  UserCtx *u = &s->user;
  DMDestroy(&u->swarm);
  PetscCall(DMCreate(PETSC_COMM_WORLD, &u->swarm));
  PetscCall(DMSetType(u->swarm, DMSWARM));
  PetscCall(DMSwarmSetType(u->swarm, DMSWARM_BASIC));
  PetscCall(RegisterParticleFields(u->swarm));
  PetscCall(DMSwarmSetLocalSizes(u->swarm, n, 0));
  u->NumberofParticles = n;
  double *fp; PetscInt *fi; PetscInt64 *fl;
  PetscCall(DMSwarmGetField(u->swarm, "position", NULL, NULL, (void **)&fp));
  memcpy(fp, pos, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(u->swarm, "position", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(u->swarm, "velocity", NULL, NULL, (void **)&fp));
  memcpy(fp, vel, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(u->swarm, "velocity", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(u->swarm, "weight", NULL, NULL, (void **)&fp));
  memcpy(fp, wgt, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(u->swarm, "weight", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(u->swarm, "P", NULL, NULL, (void **)&fp));
  memcpy(fp, P, 8 * (size_t)n);
  PetscCall(DMSwarmRestoreField(u->swarm, "P", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(u->swarm, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  for (int64_t q = 0; q < 3 * n; ++q) fi[q] = cell[q];
  PetscCall(DMSwarmRestoreField(u->swarm, "DMSwarm_CellID", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(u->swarm, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  for (int64_t q = 0; q < n; ++q) fi[q] = status[q];
  PetscCall(DMSwarmRestoreField(u->swarm, "DMSwarm_location_status", NULL, NULL, (void **)&fi));
  PetscCall(DMSwarmGetField(u->swarm, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  for (int64_t q = 0; q < n; ++q) fl[q] = pid[q];
  PetscCall(DMSwarmRestoreField(u->swarm, "DMSwarm_pid", NULL, NULL, (void **)&fl));
  return 0;
}

REF_API int ref_swarm_size(void *h, int64_t *n) {
  PetscInt m = 0;
  PetscCall(DMSwarmGetLocalSize(((RefSim *)h)->user.swarm, &m));
  *n = m;
  return 0;
}

REF_API int ref_swarm_get(void *h, double *pos, double *vel, double *wgt, double *P, int64_t *cell, int64_t *pid,
                          int64_t *status) {
  DM sw = ((RefSim *)h)->user.swarm;
  PetscInt n;
  PetscCall(DMSwarmGetLocalSize(sw, &n));
  double *fp; PetscInt *fi; PetscInt64 *fl;
  PetscCall(DMSwarmGetField(sw, "position", NULL, NULL, (void **)&fp));
  memcpy(pos, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "position", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "velocity", NULL, NULL, (void **)&fp));
  memcpy(vel, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "velocity", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "weight", NULL, NULL, (void **)&fp));
  memcpy(wgt, fp, 24 * (size_t)n);
  PetscCall(DMSwarmRestoreField(sw, "weight", NULL, NULL, (void **)&fp));
  PetscCall(DMSwarmGetField(sw, "P", NULL, NULL, (void **)&fp));
  memcpy(P, fp, 8 * (size_t)n);
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

/* The stages of one step, each the reference's own function (simulation.c:248-292):
 * 0 ResetAllParticleStatuses, 1 UpdateAllParticlePositions, 2 LocateAllParticlesInGrid_TEST,
 * 3 CheckAndRemoveLostParticles, 4 CheckAndRemoveOutOfBoundsParticles,
 * 5 InterpolateAllFieldsToSwarm, 6 ScatterAllParticleFieldsToEulerFields.
 * removed (optional) receives the local count a removal stage reports. */
REF_API int ref_stage(void *h, int stage, int64_t *removed) {
  RefSim *s = (RefSim *)h;
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
    default: return PETSC_ERR_ARG_OUTOFRANGE;
  }
  if (removed) *removed = loc;
  if (!e && minipetsc_swarm_fields_held(u->swarm))
    return minipetsc_seterr(__func__, __FILE__, __LINE__, PETSC_ERR_ARG_WRONGSTATE, "a swarm field was left held");
  return e;
}

/* PerformInitialSetup_TEST's path on one rank (simulation.c:129-175): locate, interpolate, scatter. */
REF_API int ref_initial_setup(void *h) {
  PetscCall(ref_stage(h, 2, NULL));
  PetscCall(ref_stage(h, 5, NULL));
  return ref_stage(h, 6, NULL);
}

/* One iteration of AdvanceSimulation_TEST's loop (simulation.c:248-292); removed[0], [1]: the
 * LOST and out-of-bounds counts. */
REF_API int ref_step(void *h, int64_t *removed) {
  int64_t lost = 0, oob = 0;
  PetscCall(ref_stage(h, 0, NULL));
  PetscCall(ref_stage(h, 1, NULL));
  PetscCall(ref_stage(h, 2, NULL));
  PetscCall(ref_stage(h, 3, &lost));
  PetscCall(ref_stage(h, 4, &oob));
  PetscCall(ref_stage(h, 5, NULL));
  PetscCall(ref_stage(h, 6, NULL));
  if (removed) { removed[0] = lost; removed[1] = oob; }
  return 0;
}

/* ParticleCount and the P average (node-sized [KM+1][JM+1][IM+1]) after a scatter. */
REF_API int ref_get_scattered(void *h, double *count, double *P) {
  RefSim *s = (RefSim *)h;
  const PetscInt Nn = minipetsc_vec_length(s->user.P);
  memcpy(count, minipetsc_vec_data(s->user.ParticleCount), (size_t)Nn * sizeof(double));
  memcpy(P, minipetsc_vec_data(s->user.P), (size_t)Nn * sizeof(double));
  return 0;
}
