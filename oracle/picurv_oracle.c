/*
 * picurv_oracle.c -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
 *
 * CPU restatement of PICurv's particle hot path, the checker for the CUDA path.
 * Built with -O2 -ffp-contract=off so that no a*b+c is fused, matching the
 * reference objects (compiled at -O0 without FMA).  Operation order is literal.
 * Citations are file:line within the reference project (VishalKandala/fdf).
 */
#include "picurv_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_MAX_TRAVERSAL 1000           /* walkingsearch.c:10 */
#define O_DISTANCE_THRESHOLD 1e-11     /* walkingsearch.c:11 */
#define O_REPEAT_COUNT_THRESHOLD 5     /* walkingsearch.c:12 */
#define O_INTERP_DIST_TOL 1e-14        /* ParticleSwarm.c:5  */
#define O_BBOX_TOLERANCE 1e-6          /* grid.c:6           */

/* PETSc's PetscMin/PetscMax macros (petscmath.h): a<b ? a : b and a<b ? b : a. */
static inline double o_min(double a, double b) { return (a < b) ? a : b; }
static inline double o_max(double a, double b) { return (a < b) ? b : a; }

static inline const double *node_at(const OGrid *g, int64_t i, int64_t j, int64_t k) {
  return g->coor + 3 * ((k * (g->JM + 1) + j) * (g->IM + 1) + i);
}

/* walkingsearch.c:25-59 -- mean of the 12 edge lengths. */
int o_GetCellCharacteristicSize(const OCell *cell, double *cellSize) {
  if (!cell || !cellSize) return O_ERR_ARG_NULL;
  static const int edges[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                   {6, 7}, {7, 4}, {0, 7}, {1, 6}, {2, 5}, {3, 4}};
  double total = 0.0;
  for (int i = 0; i < 12; i++) {
    OCmpnts A = cell->vertices[edges[i][0]];
    OCmpnts B = cell->vertices[edges[i][1]];
    double dx = B.x - A.x, dy = B.y - A.y, dz = B.z - A.z;
    double len = sqrt(dx * dx + dy * dy + dz * dz);
    total += len;
  }
  *cellSize = total / 12.0;
  return 0;
}

/* walkingsearch.c:102-227 -- signed distance to the plane of face (v1,v2,v3,v4). */
int o_ComputeSignedDistanceToPlane(OCmpnts v1, OCmpnts v2, OCmpnts v3, OCmpnts v4,
                                   OCmpnts cc, OCmpnts p, double *d_signed, double threshold) {
  if (!d_signed) return O_ERR_ARG_NULL;
  double e1x = v2.x - v1.x, e1y = v2.y - v1.y, e1z = v2.z - v1.z;
  double e2x = v4.x - v1.x, e2y = v4.y - v1.y, e2z = v4.z - v1.z;
  double nxi = e1y * e2z - e1z * e2y;
  double nyi = e1z * e2x - e1x * e2z;
  double nzi = e1x * e2y - e1y * e2x;
  double mag = sqrt(nxi * nxi + nyi * nyi + nzi * nzi);
  if (mag < 1.0e-12) return O_ERR_USER;                    /* :147-155 */
  double fcx = 0.25 * (v1.x + v2.x + v3.x + v4.x);
  double fcy = 0.25 * (v1.y + v2.y + v3.y + v4.y);
  double fcz = 0.25 * (v1.z + v2.z + v3.z + v4.z);
  double tx = cc.x - fcx, ty = cc.y - fcy, tz = cc.z - fcz;
  double dot = nxi * tx + nyi * ty + nzi * tz;
  double nx = nxi, ny = nyi, nz = nzi;
  if (dot > 1.0e-9) { nx = -nxi; ny = -nyi; nz = -nzi; }   /* :181-185 */
  nx /= mag; ny /= mag; nz /= mag;
  double px = fcx - p.x, py = fcy - p.y, pz = fcz - p.z;
  double d = px * nx + py * ny + pz * nz;
  if (fabs(d) < threshold) d = 0.0;                         /* :218-221 */
  *d_signed = d;
  return 0;
}

/* walkingsearch.c:271-389 -- the six faces, in the reference's evaluation order. */
int o_CalculateDistancesToCellFaces(OCmpnts p, const OCell *cell, double *d, double threshold) {
  if (!cell || !d) return O_ERR_ARG_NULL;
  OCmpnts cc = {0.0, 0.0, 0.0};
  for (int i = 0; i < 8; ++i) {
    cc.x += cell->vertices[i].x; cc.y += cell->vertices[i].y; cc.z += cell->vertices[i].z;
  }
  cc.x /= 8.0; cc.y /= 8.0; cc.z /= 8.0;
  const OCmpnts *v = cell->vertices;
  int ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[0], v[3], v[2], v[1], cc, p, &d[O_BACK], threshold))) return ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[4], v[7], v[6], v[5], cc, p, &d[O_FRONT], threshold))) return ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[0], v[1], v[6], v[7], cc, p, &d[O_BOTTOM], threshold))) return ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[3], v[4], v[5], v[2], cc, p, &d[O_TOP], threshold))) return ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[0], v[7], v[4], v[3], cc, p, &d[O_LEFT], threshold))) return ierr;
  if ((ierr = o_ComputeSignedDistanceToPlane(v[1], v[2], v[5], v[6], cc, p, &d[O_RIGHT], threshold))) return ierr;
  return 0;
}

/* walkingsearch.c:407-462 -- 0 inside, 1/2/3 on 1/2/>=3 faces (and outside others), -1 outside. */
int o_DeterminePointPosition(const double *d, int64_t *result) {
  if (!d || !result) return O_ERR_ARG_NULL;
  int isInside = 1, isOnBoundary = 0;
  int64_t count = 0;
  for (int i = 0; i < O_NUM_FACES; i++) {
    if (d[i] < 0.0) isInside = 0;
    if (d[i] == 0.0) { isOnBoundary = 1; count++; }
  }
  if (isInside) *result = 0;
  else if (isOnBoundary) {
    if (count == 1) *result = 1;
    else if (count == 2) *result = 2;
    else *result = 3;
  } else *result = -1;
  return 0;
}

/* walkingsearch.c:521-549 -- vertex numbering of the walking search. */
int o_GetCellVerticesFromGrid(const OGrid *g, int64_t i, int64_t j, int64_t k, OCell *cell) {
  if (!g || !cell) return O_ERR_ARG_NULL;
  const int64_t off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                             {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}};
  for (int c = 0; c < 8; ++c) {
    const double *q = node_at(g, i + off[c][0], j + off[c][1], k + off[c][2]);
    cell->vertices[c].x = q[0]; cell->vertices[c].y = q[1]; cell->vertices[c].z = q[2];
  }
  return 0;
}

/* walkingsearch.c:811-859 -- threshold scaled by the cell size, then classify. */
int o_EvaluateParticlePosition(const OCell *cell, double *d, OCmpnts p, int64_t *position, double threshold) {
  if (!cell || !position) return O_ERR_ARG_NULL;
  double cellSize;
  int ierr = o_GetCellCharacteristicSize(cell, &cellSize);
  if (ierr) return ierr;
  double cellThreshold = threshold * cellSize;
  ierr = o_CalculateDistancesToCellFaces(p, cell, d, cellThreshold);
  if (ierr) return ierr;   /* CHKERRQ at :838 returns before the skip branch at :843 */
  return o_DeterminePointPosition(d, position);
}

/* walkingsearch.c:882-959 -- k first, then i, then j; "else if" priority; no clamping. */
int o_UpdateCellIndicesBasedOnDistancesTEST(const double d[6], int64_t *idx, int64_t *idy, int64_t *idz) {
  if (!d || !idx || !idy || !idz) return O_ERR_ARG_NULL;
  if (d[O_FRONT] < 0.0) (*idz) += 1;
  else if (d[O_BACK] < 0.0) (*idz) -= 1;
  if (d[O_LEFT] < 0.0) (*idx) -= 1;
  else if (d[O_RIGHT] < 0.0) (*idx) += 1;
  if (d[O_BOTTOM] < 0.0) (*idy) -= 1;
  else if (d[O_TOP] < 0.0) (*idy) += 1;
  return 0;
}

/* ParticleSwarm.c:1010-1047 -- clamps d in place, then the three ratios. */
int o_UpdateParticleWeights(double *d, double w[3]) {
  if (!d || !w) return O_ERR_ARG_NULL;
  for (int i = O_LEFT; i < O_NUM_FACES; i++)
    if (d[i] <= O_INTERP_DIST_TOL) d[i] = O_INTERP_DIST_TOL;
  w[0] = d[O_LEFT] / (d[O_LEFT] + d[O_RIGHT]);
  w[1] = d[O_BOTTOM] / (d[O_BOTTOM] + d[O_TOP]);
  w[2] = d[O_BACK] / (d[O_FRONT] + d[O_BACK]);
  return 0;
}

/* walkingsearch.c:650-708 on one rank: the ghosted node range is every node, so a
 * cell is "local" iff 0 <= idx < IM (and likewise j, k). */
static int o_cell_within_local_grid(const OGrid *g, int64_t i, int64_t j, int64_t k) {
  return i >= 0 && i < g->IM && j >= 0 && j < g->JM && k >= 0 && k < g->KM;
}

/* walkingsearch.c:1094-1242 (with :571-629 for the start cell and :1026-1071 for the
 * owner, which on one rank owns every cell, setup.c:679-765). */
int o_LocateParticleOrFindMigrationTarget(const OGrid *g, const double loc[3], int64_t cell[3],
                                          double weights[3], int64_t *status, int64_t *steps_out) {
  int64_t idx, idy, idz, steps = 0;
  int concluded = 0;
  int64_t repeated = 0;
  int64_t prevIdx = INT64_MIN, prevIdy = INT64_MIN, prevIdz = INT64_MIN;
  int64_t last_position = -999;
  OCmpnts p = {loc[0], loc[1], loc[2]};
  int ierr;

  /* InitializeTraversalParameters :571-629 */
  if (cell[0] >= 0 && cell[1] >= 0 && cell[2] >= 0 &&
      o_cell_within_local_grid(g, cell[0], cell[1], cell[2])) {
    idx = cell[0]; idy = cell[1]; idz = cell[2];
  } else {
    idx = 0; idy = 0; idz = 0;   /* local corner (xs, ys, zs) of the one rank */
  }

  while (!concluded && steps < O_MAX_TRAVERSAL) {
    steps++;
    if (idx < 0 || idx >= g->IM || idy < 0 || idy >= g->JM || idz < 0 || idz >= g->KM) {
      idx = -1;                                  /* :1127-1132 */
      break;
    }
    if (!o_cell_within_local_grid(g, idx, idy, idz)) {   /* :1137-1146, never on one rank */
      concluded = 1;
      continue;
    }
    if (idx == prevIdx && idy == prevIdy && idz == prevIdz) {   /* :1149-1185 */
      repeated++;
      if (repeated > O_REPEAT_COUNT_THRESHOLD) {
        if (last_position >= 1) {
          OCell fc; double fd[6]; int64_t fpos;
          o_GetCellVerticesFromGrid(g, idx, idy, idz, &fc);
          ierr = o_EvaluateParticlePosition(&fc, fd, p, &fpos, O_DISTANCE_THRESHOLD);
          if (ierr == 0) { o_UpdateParticleWeights(fd, weights); concluded = 1; }
          else { idx = -1; concluded = 1; }
        } else {
          idx = -1; concluded = 1;
        }
        if (concluded) continue;
      }
    } else {
      repeated = 0;
    }
    prevIdx = idx; prevIdy = idy; prevIdz = idz;

    OCell c; double d[6]; int64_t position;
    o_GetCellVerticesFromGrid(g, idx, idy, idz, &c);
    ierr = o_EvaluateParticlePosition(&c, d, p, &position, O_DISTANCE_THRESHOLD);
    if (ierr) { if (steps_out) *steps_out = steps; return ierr; }   /* CHKERRQ :1193 */
    last_position = position;
    if (position >= 0) {
      concluded = 1;
      o_UpdateParticleWeights(d, weights);
    } else {
      o_UpdateCellIndicesBasedOnDistancesTEST(d, &idx, &idy, &idz);
    }
  }

  if (idx == -1 || (!concluded && steps >= O_MAX_TRAVERSAL)) {   /* :1206-1213 */
    *status = O_LOST;
    cell[0] = cell[1] = cell[2] = -1;
  } else {
    /* FindOwnerOfCell on one rank: every in-range cell is owned by rank 0. */
    cell[0] = idx; cell[1] = idy; cell[2] = idz;
    if (o_cell_within_local_grid(g, idx, idy, idz)) *status = O_ACTIVE_AND_LOCATED;
    else { *status = O_LOST; cell[0] = cell[1] = cell[2] = -1; }
  }
  if (steps_out) *steps_out = steps;
  return 0;
}

/* ParticleMotion.c:2149-2176 */
void o_ResetAllParticleStatuses(OSwarm *s) {
  for (int64_t p = 0; p < s->n; ++p)
    if (s->status[p] == O_ACTIVE_AND_LOCATED) s->status[p] = O_NEEDS_LOCATION;
}

/* ParticleMotion.c:19-29, 38-95 -- x += v*dt per component. */
void o_UpdateAllParticlePositions(OSwarm *s, double dt, int nthreads) {
  (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t p = 0; p < s->n; p++) {
    s->pos[3 * p + 0] += s->vel[3 * p + 0] * dt;
    s->pos[3 * p + 1] += s->vel[3 * p + 1] * dt;
    s->pos[3 * p + 2] += s->vel[3 * p + 2] * dt;
  }
}

/* ParticleMotion.c:1931-2135 on one rank: one pass, no migration. Particles already
 * ACTIVE_AND_LOCATED are skipped (:1992); all others walk (both CASE branches walk on
 * one rank because GuessParticleOwnerWithBBox can only answer self or none). */
int o_LocateAllParticlesInGrid(const OGrid *g, OSwarm *s, int nthreads, int64_t *evals_out) {
  int64_t evals = 0;
  int err = 0;
  (void)nthreads;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : evals) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t p = 0; p < s->n; p++) {
    if (s->status[p] == O_ACTIVE_AND_LOCATED) continue;
    int64_t st = s->status[p], steps = 0;
    int e = o_LocateParticleOrFindMigrationTarget(g, &s->pos[3 * p], &s->cell[3 * p],
                                                  &s->weight[3 * p], &st, &steps);
    evals += steps;
    if (e) {
#pragma omp atomic write
      err = e;
    }
    s->status[p] = st;
  }
  if (evals_out) *evals_out = evals;
  return err;
}

/* DMSwarmRemovePointAtIndex: the last point is copied into slot p, size shrinks by one. */
static void o_swarm_remove_at(OSwarm *s, int64_t p) {
  int64_t last = s->n - 1;
  if (p != last) {
    memcpy(&s->pos[3 * p], &s->pos[3 * last], 3 * sizeof(double));
    memcpy(&s->vel[3 * p], &s->vel[3 * last], 3 * sizeof(double));
    memcpy(&s->weight[3 * p], &s->weight[3 * last], 3 * sizeof(double));
    memcpy(&s->cell[3 * p], &s->cell[3 * last], 3 * sizeof(int64_t));
    s->P[p] = s->P[last];
    s->pid[p] = s->pid[last];
    s->status[p] = s->status[last];
  }
  s->n = last;
}

/* ParticleMotion.c:532-625 -- backward loop, remove status == LOST. */
void o_CheckAndRemoveLostParticles(OSwarm *s, int64_t *removed) {
  int64_t r = 0;
  for (int64_t p = s->n - 1; p >= 0; p--)
    if (s->status[p] == O_LOST) { o_swarm_remove_at(s, p); r++; }
  if (removed) *removed = r;
}

/* grid.c:762-883 on one rank: min/max over every node, widened by 1e-6. */
void o_ComputeLocalBoundingBox(const OGrid *g, double bmin[3], double bmax[3]) {
  int64_t nn = (g->IM + 1) * (g->JM + 1) * (g->KM + 1);
  for (int c = 0; c < 3; c++) { bmin[c] = 1.7976931348623157e308; bmax[c] = -1.7976931348623157e308; }
  for (int64_t q = 0; q < nn; q++)
    for (int c = 0; c < 3; c++) {
      double v = g->coor[3 * q + c];
      if (v < bmin[c]) bmin[c] = v;
      if (v > bmax[c]) bmax[c] = v;
    }
  for (int c = 0; c < 3; c++) { bmin[c] = bmin[c] - O_BBOX_TOLERANCE; bmax[c] = bmax[c] + O_BBOX_TOLERANCE; }
}

/* ParticleMotion.c:283-383 with IsParticleInBox :106-110. */
void o_CheckAndRemoveOutOfBoundsParticles(const OGrid *g, OSwarm *s, int64_t *removed) {
  double bmin[3], bmax[3];
  o_ComputeLocalBoundingBox(g, bmin, bmax);
  int64_t r = 0;
  for (int64_t p = s->n - 1; p >= 0; p--) {
    const double *x = &s->pos[3 * p];
    int inside = x[0] >= bmin[0] && x[0] <= bmax[0] && x[1] >= bmin[1] && x[1] <= bmax[1] &&
                 x[2] >= bmin[2] && x[2] <= bmax[2];
    if (!inside) { o_swarm_remove_at(s, p); r++; }
  }
  if (removed) *removed = r;
}

/* interpolation.c:598-679 -- each node = mean of its valid adjacent cells (k, j, i loops
 * over offsets -1..0). */
void o_InterpolateFieldFromCenterToCorner_Vector(const OGrid *g, const double *ucat, double *corner, int nthreads) {
  const int64_t mx = g->IM + 1, my = g->JM + 1, mz = g->KM + 1;
  (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t k = 0; k < mz; k++)
    for (int64_t j = 0; j < my; j++)
      for (int64_t i = 0; i < mx; i++) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        int64_t count = 0;
        for (int64_t dk = -1; dk <= 0; dk++)
          for (int64_t dj = -1; dj <= 0; dj++)
            for (int64_t di = -1; di <= 0; di++) {
              int64_t ck = k + dk, cj = j + dj, ci = i + di;
              if (ci >= 0 && ci < mx - 1 && cj >= 0 && cj < my - 1 && ck >= 0 && ck < mz - 1) {
                const double *v = ucat + 3 * ((ck * my + cj) * mx + ci);
                sx += v[0]; sy += v[1]; sz += v[2];
                count++;
              }
            }
        double *o = corner + 3 * ((k * my + j) * mx + i);
        if (count > 0) {
          o[0] = sx / (double)count; o[1] = sy / (double)count; o[2] = sz / (double)count;
        } else {
          o[0] = 0.0; o[1] = 0.0; o[2] = 0.0;
        }
      }
}

/* interpolation.c:839-864 (weights with PetscMax/PetscMin clamping) and :957-1042. */
void o_TrilinearInterpolation_Vector(const OGrid *g, const double *corner, int64_t i, int64_t j, int64_t k,
                                     double a1, double a2, double a3, double out[3]) {
  const int64_t mx = g->IM + 1, my = g->JM + 1;
  a1 = o_max(0.0, o_min(1.0, a1));
  a2 = o_max(0.0, o_min(1.0, a2));
  a3 = o_max(0.0, o_min(1.0, a3));
  const double oa1 = 1.0 - a1, oa2 = 1.0 - a2, oa3 = 1.0 - a3;
  double w[8];
  w[0] = oa1 * oa2 * oa3; w[1] = a1 * oa2 * oa3; w[2] = oa1 * a2 * oa3; w[3] = a1 * a2 * oa3;
  w[4] = oa1 * oa2 * a3;  w[5] = a1 * oa2 * a3;  w[6] = oa1 * a2 * a3;  w[7] = a1 * a2 * a3;
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  double sumW = 0.0, ax = 0.0, ay = 0.0, az = 0.0;
  for (int c = 0; c < 8; c++) {
    const double *v = corner + 3 * (((k + off[c][2]) * my + (j + off[c][1])) * mx + (i + off[c][0]));
    ax += w[c] * v[0];
    ay += w[c] * v[1];
    az += w[c] * v[2];
    sumW += w[c];
  }
  if (sumW > 1.0e-14) { out[0] = ax / sumW; out[1] = ay / sumW; out[2] = az / sumW; }
  else { out[0] = 0.0; out[1] = 0.0; out[2] = 0.0; }
}

/* interpolation.c:1205-1399, stage 2: stencil guard :1356-1372, then trilinear. */
void o_InterpolateEulerFieldToSwarm(const OGrid *g, const double *corner, OSwarm *s, int nthreads) {
  (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t p = 0; p < s->n; p++) {
    int64_t i = s->cell[3 * p], j = s->cell[3 * p + 1], k = s->cell[3 * p + 2];
    /* gxs + gxm - 1 = IM on one rank (gxm = IM+1 nodes) */
    if (i < 0 || i >= g->IM || j < 0 || j >= g->JM || k < 0 || k >= g->KM) {
      s->vel[3 * p] = 0.0; s->vel[3 * p + 1] = 0.0; s->vel[3 * p + 2] = 0.0;
      continue;
    }
    o_TrilinearInterpolation_Vector(g, corner, i, j, k, s->weight[3 * p], s->weight[3 * p + 1],
                                    s->weight[3 * p + 2], &s->vel[3 * p]);
  }
}

/* interpolation.c:2063-2116 via AccumulateParticleField :1838-1923,
 * CalculateParticleCountPerCell ParticleMotion.c:931-1067 and
 * NormalizeGridVectorByCount interpolation.c:1943-2036, for the field "P". */
void o_ScatterParticleFieldToEulerField_P(const OGrid *g, const OSwarm *s, double *count, double *avg) {
  const int64_t gxm = g->IM + 1, gym = g->JM + 1, gzm = g->KM + 1;
  const int64_t nn = gxm * gym * gzm;
  double *sum = (double *)calloc((size_t)nn, sizeof(double));
  for (int64_t q = 0; q < nn; q++) count[q] = 0.0;
  for (int64_t p = 0; p < s->n; ++p) {   /* AccumulateParticleField */
    int64_t i = s->cell[3 * p], j = s->cell[3 * p + 1], k = s->cell[3 * p + 2];
    if (i >= 0 && i < gxm && j >= 0 && j < gym && k >= 0 && k < gzm)
      sum[(k * gym + j) * gxm + i] += s->P[p];
  }
  for (int64_t p = 0; p < s->n; p++) {   /* CalculateParticleCountPerCell */
    int64_t i = s->cell[3 * p], j = s->cell[3 * p + 1], k = s->cell[3 * p + 2];
    if (i >= 0 && i < gxm && j >= 0 && j < gym && k >= 0 && k < gzm)
      count[(k * gym + j) * gxm + i] += 1.0;
  }
  for (int64_t q = 0; q < nn; q++)       /* NormalizeGridVectorByCount */
    avg[q] = (count[q] > 0.5) ? sum[q] / count[q] : 0.0;
  free(sum);
}

/* The face deposit is defined with a fixed summation order: particles in
 * ascending (linear cell id i + IM*(j + JM*k), PID) order, each face summing its
 * contributions in that order from a starting 0.0.  A face's lower cell precedes
 * its upper cell in that order, so every face adds its lower cell's particles
 * (weight a) first and its upper cell's (weight 1-a) second. */
/* The (cell, PID) order of the particles with a cell: a counting sort by cell (start[c] ..
 * start[c + 1] are cell c's entries of idx), each cell's entries then in ascending PID (and slot).
 * Returns the number of particles placed, or -1 when out of memory. */
static int64_t o_cell_order(const OGrid *g, const OSwarm *s, int64_t *start, int64_t *idx) {
  const int64_t IM = g->IM, JM = g->JM, KM = g->KM, Nc = IM * JM * KM;
  for (int64_t c = 0; c <= Nc; c++) start[c] = 0;
  for (int64_t p = 0; p < s->n; p++) {
    int64_t i = s->cell[3 * p], j = s->cell[3 * p + 1], k = s->cell[3 * p + 2];
    if (i < 0 || i >= IM || j < 0 || j >= JM || k < 0 || k >= KM) continue;
    start[(k * JM + j) * IM + i + 1]++;
  }
  for (int64_t c = 0; c < Nc; c++) start[c + 1] += start[c];
  int64_t *fill = (int64_t *)malloc((size_t)(Nc > 0 ? Nc : 1) * sizeof(int64_t));
  if (!fill) return -1;
  memcpy(fill, start, (size_t)Nc * sizeof(int64_t));
  for (int64_t p = 0; p < s->n; p++) {   /* ascending slot within each cell */
    int64_t i = s->cell[3 * p], j = s->cell[3 * p + 1], k = s->cell[3 * p + 2];
    if (i < 0 || i >= IM || j < 0 || j >= JM || k < 0 || k >= KM) continue;
    idx[fill[(k * JM + j) * IM + i]++] = p;
  }
  free(fill);
  const int64_t *pid = s->pid;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t c = 0; c < Nc; c++) {     /* then ascending PID (insertion sort: a few per cell) */
    for (int64_t a = start[c] + 1; a < start[c + 1]; a++) {
      const int64_t v = idx[a];
      int64_t b = a - 1;
      while (b >= start[c] && pid[idx[b]] > pid[v]) { idx[b + 1] = idx[b]; b--; }
      idx[b + 1] = v;
    }
  }
  return start[Nc];
}

/* One face's sum in the deposit's order: its lower cell's particles (weight a, the upper-face
 * fraction a * V/3) from 0.0, then its upper cell's (the lower-face fraction (1 - a) * V/3);
 * a side outside the grid contributes nothing.  comp: the weight component (0 i, 1 j, 2 k). */
static void o_face_sum(const OSwarm *s, const int64_t *start, const int64_t *idx, int64_t lower, int64_t upper,
                       int comp, double third, double *vol, double *mom3, double *absum) {
  double v = 0.0, ab = 0.0, m0 = 0.0, m1 = 0.0, m2 = 0.0;
  for (int side = 0; side < 2; side++) {
    const int64_t c = side == 0 ? lower : upper;
    if (c < 0) continue;
    for (int64_t q = start[c]; q < start[c + 1]; q++) {
      const int64_t p = idx[q];
      const double a = s->weight[3 * p + comp];
      const double frac = side == 0 ? a * third : (1.0 - a) * third;
      v += frac;
      ab += fabs(frac);
      if (mom3) {
        const double *u = &s->vel[3 * p];
        m0 += frac * u[0]; m1 += frac * u[1]; m2 += frac * u[2];
      }
    }
  }
  *vol = v;
  if (absum) *absum = ab;
  if (mom3) { mom3[0] = m0; mom3[1] = m1; mom3[2] = m2; }
}

void o_DepositParticlesToFaces(const OGrid *g, const OSwarm *s, double volume,
                               double *fi, double *fj, double *fk,
                               double *mom_i, double *mom_j, double *mom_k,
                               double *abs_i, double *abs_j, double *abs_k) {
  const int64_t IM = g->IM, JM = g->JM, KM = g->KM, Nc = IM * JM * KM;
  const double third = volume / 3.0;
  int64_t *start = (int64_t *)malloc((size_t)(Nc + 1) * sizeof(int64_t));
  int64_t *idx = (int64_t *)malloc((size_t)(s->n > 0 ? s->n : 1) * sizeof(int64_t));
  if (!start || !idx || o_cell_order(g, s, start, idx) < 0) { free(start); free(idx); return; }
  /* i-face (i, j, k): cells (i-1, j, k) and (i, j, k) */
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < (IM + 1) * JM * KM; f++) {
    const int64_t i = f % (IM + 1), jk = f / (IM + 1);
    const int64_t c = jk * IM + i;
    o_face_sum(s, start, idx, i > 0 ? c - 1 : -1, i < IM ? c : -1, 0, third, &fi[f], mom_i ? &mom_i[3 * f] : NULL,
               abs_i ? &abs_i[f] : NULL);
  }
  /* j-face (i, j, k): cells (i, j-1, k) and (i, j, k) */
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < IM * (JM + 1) * KM; f++) {
    const int64_t i = f % IM, j = (f / IM) % (JM + 1), k = f / (IM * (JM + 1));
    const int64_t c = (k * JM + j) * IM + i;
    o_face_sum(s, start, idx, j > 0 ? c - IM : -1, j < JM ? c : -1, 1, third, &fj[f], mom_j ? &mom_j[3 * f] : NULL,
               abs_j ? &abs_j[f] : NULL);
  }
  /* k-face (i, j, k): cells (i, j, k-1) and (i, j, k) */
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < IM * JM * (KM + 1); f++) {
    const int64_t k = f / (IM * JM);
    o_face_sum(s, start, idx, k > 0 ? f - IM * JM : -1, k < KM ? f : -1, 2, third, &fk[f],
               mom_k ? &mom_k[3 * f] : NULL, abs_k ? &abs_k[f] : NULL);
  }
  free(start);
  free(idx);
}

/* simulation.c:240-311 (one step, one rank, steady ucat). */
int o_AdvanceStep(const OGrid *g, const double *ucat, double *corner, OSwarm *s, double dt,
                  double *count, double *avg, int nthreads, OStepInfo *info) {
  OStepInfo loc = {0, 0, 0, s->n};
  o_ResetAllParticleStatuses(s);
  o_UpdateAllParticlePositions(s, dt, nthreads);
  int err = o_LocateAllParticlesInGrid(g, s, nthreads, &loc.evals);
  if (err) { if (info) *info = loc; return err; }
  o_CheckAndRemoveLostParticles(s, &loc.removed_lost);
  o_CheckAndRemoveOutOfBoundsParticles(g, s, &loc.removed_oob);
  o_InterpolateFieldFromCenterToCorner_Vector(g, ucat, corner, nthreads);
  o_InterpolateEulerFieldToSwarm(g, corner, s, nthreads);
  if (count && avg) o_ScatterParticleFieldToEulerField_P(g, s, count, avg);
  if (info) *info = loc;
  return 0;
}

/* simulation.c:129-175 without inlet re-seeding: locate, interpolate, scatter.
 * LOST particles are not removed here (the reference removes them in step 1). */
int o_InitialSetup(const OGrid *g, const double *ucat, double *corner, OSwarm *s,
                   double *count, double *avg, int nthreads, OStepInfo *info) {
  OStepInfo loc = {0, 0, 0, s->n};
  int err = o_LocateAllParticlesInGrid(g, s, nthreads, &loc.evals);
  if (err) { if (info) *info = loc; return err; }
  o_InterpolateFieldFromCenterToCorner_Vector(g, ucat, corner, nthreads);
  o_InterpolateEulerFieldToSwarm(g, corner, s, nthreads);
  if (count && avg) o_ScatterParticleFieldToEulerField_P(g, s, count, avg);
  if (info) *info = loc;
  return 0;
}

/* ======================================================================== */
/* The Eulerian input of the path: face metrics, the Jacobian, Contra2Cart.  */
/* ======================================================================== */

static inline int64_t o_nidx(const OGrid *g, int64_t i, int64_t j, int64_t k) {
  return (k * (g->JM + 1) + j) * (g->IM + 1) + i;
}

/* copy one node's 3-vector */
static inline void o_cp3(double *a, int64_t dst, int64_t src) {
  a[3 * dst] = a[3 * src]; a[3 * dst + 1] = a[3 * src + 1]; a[3 * dst + 2] = a[3 * src + 2];
}

/* Metric.c:286-460.  One rank owns every node: xs = ys = zs = 0, xe = mx, ye = my, ze = mz. */
void o_ComputeFaceMetrics(const OGrid *g, double *csi, double *eta, double *zet) {
  const int64_t mx = g->IM + 1, my = g->JM + 1, mz = g->KM + 1, nn = mx * my * mz;
  memset(csi, 0, (size_t)(3 * nn) * sizeof(double));
  memset(eta, 0, (size_t)(3 * nn) * sizeof(double));
  memset(zet, 0, (size_t)(3 * nn) * sizeof(double));
#define P_(c, ii, jj, kk) (node_at(g, (ii), (jj), (kk))[c])
  for (int64_t k = 1; k < mz; ++k)            /* Csi :325-341 */
    for (int64_t j = 1; j < my; ++j)
      for (int64_t i = 0; i < mx; ++i) {
        double de[3], dz[3];
        for (int c = 0; c < 3; ++c) {
          de[c] = 0.5 * (P_(c, i, j, k) + P_(c, i, j, k - 1) - P_(c, i, j - 1, k) - P_(c, i, j - 1, k - 1));
          dz[c] = 0.5 * (P_(c, i, j - 1, k) + P_(c, i, j, k) - P_(c, i, j - 1, k - 1) - P_(c, i, j, k - 1));
        }
        double *o = csi + 3 * o_nidx(g, i, j, k);
        o[0] = de[1] * dz[2] - de[2] * dz[1];
        o[1] = de[2] * dz[0] - de[0] * dz[2];
        o[2] = de[0] * dz[1] - de[1] * dz[0];
      }
  for (int64_t k = 1; k < mz; ++k)            /* Eta :344-360 */
    for (int64_t j = 0; j < my; ++j)
      for (int64_t i = 1; i < mx; ++i) {
        double dx[3], dz[3];
        for (int c = 0; c < 3; ++c) {
          dx[c] = 0.5 * (P_(c, i, j, k) + P_(c, i, j, k - 1) - P_(c, i - 1, j, k) - P_(c, i - 1, j, k - 1));
          dz[c] = 0.5 * (P_(c, i, j, k) + P_(c, i - 1, j, k) - P_(c, i, j, k - 1) - P_(c, i - 1, j, k - 1));
        }
        double *o = eta + 3 * o_nidx(g, i, j, k);
        o[0] = dz[1] * dx[2] - dz[2] * dx[1];
        o[1] = dz[2] * dx[0] - dz[0] * dx[2];
        o[2] = dz[0] * dx[1] - dz[1] * dx[0];
      }
  for (int64_t k = 0; k < mz; ++k)            /* Zet :363-379 */
    for (int64_t j = 1; j < my; ++j)
      for (int64_t i = 1; i < mx; ++i) {
        double dx[3], de[3];
        for (int c = 0; c < 3; ++c) {
          dx[c] = 0.5 * (P_(c, i, j, k) + P_(c, i, j - 1, k) - P_(c, i - 1, j, k) - P_(c, i - 1, j - 1, k));
          de[c] = 0.5 * (P_(c, i, j, k) + P_(c, i - 1, j, k) - P_(c, i, j - 1, k) - P_(c, i - 1, j - 1, k));
        }
        double *o = zet + 3 * o_nidx(g, i, j, k);
        o[0] = dx[1] * de[2] - dx[2] * de[1];
        o[1] = dx[2] * de[0] - dx[0] * de[2];
        o[2] = dx[0] * de[1] - dx[1] * de[0];
      }
#undef P_
  /* boundary extrapolation :383-452, in the reference's order: i, then j, then k */
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t j = 0; j < my; ++j)
      if (1 < mx) { o_cp3(eta, o_nidx(g, 0, j, k), o_nidx(g, 1, j, k)); o_cp3(zet, o_nidx(g, 0, j, k), o_nidx(g, 1, j, k)); }
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t j = 0; j < my; ++j)
      if (mx - 2 >= 0) {
        o_cp3(eta, o_nidx(g, mx - 1, j, k), o_nidx(g, mx - 2, j, k));
        o_cp3(zet, o_nidx(g, mx - 1, j, k), o_nidx(g, mx - 2, j, k));
      }
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t i = 0; i < mx; ++i)
      if (1 < my) { o_cp3(csi, o_nidx(g, i, 0, k), o_nidx(g, i, 1, k)); o_cp3(zet, o_nidx(g, i, 0, k), o_nidx(g, i, 1, k)); }
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t i = 0; i < mx; ++i)
      if (my - 2 >= 0) {
        o_cp3(csi, o_nidx(g, i, my - 1, k), o_nidx(g, i, my - 2, k));
        o_cp3(zet, o_nidx(g, i, my - 1, k), o_nidx(g, i, my - 2, k));
      }
  for (int64_t j = 0; j < my; ++j)
    for (int64_t i = 0; i < mx; ++i)
      if (1 < mz) { o_cp3(csi, o_nidx(g, i, j, 0), o_nidx(g, i, j, 1)); o_cp3(eta, o_nidx(g, i, j, 0), o_nidx(g, i, j, 1)); }
  for (int64_t j = 0; j < my; ++j)
    for (int64_t i = 0; i < mx; ++i)
      if (mz - 2 >= 0) {
        o_cp3(csi, o_nidx(g, i, j, mz - 1), o_nidx(g, i, j, mz - 2));
        o_cp3(eta, o_nidx(g, i, j, mz - 1), o_nidx(g, i, j, mz - 2));
      }
}

/* Metric.c:491-600. */
int o_ComputeCellCenteredJacobianInverse(const OGrid *g, double *aj) {
  const int64_t mx = g->IM + 1, my = g->JM + 1, mz = g->KM + 1, nn = mx * my * mz;
  memset(aj, 0, (size_t)nn * sizeof(double));
#define P_(c, ii, jj, kk) (node_at(g, (ii), (jj), (kk))[c])
  for (int64_t k = 1; k < mz; ++k)
    for (int64_t j = 1; j < my; ++j)
      for (int64_t i = 1; i < mx; ++i) {
        double dxi[3], deta[3], dzeta[3];
        for (int c = 0; c < 3; ++c) {
          dxi[c] = 0.25 * ((P_(c, i, j, k) + P_(c, i, j - 1, k) + P_(c, i, j, k - 1) + P_(c, i, j - 1, k - 1)) -
                           (P_(c, i - 1, j, k) + P_(c, i - 1, j - 1, k) + P_(c, i - 1, j, k - 1) + P_(c, i - 1, j - 1, k - 1)));
          deta[c] = 0.25 * ((P_(c, i, j, k) + P_(c, i - 1, j, k) + P_(c, i, j, k - 1) + P_(c, i - 1, j, k - 1)) -
                            (P_(c, i, j - 1, k) + P_(c, i - 1, j - 1, k) + P_(c, i, j - 1, k - 1) + P_(c, i - 1, j - 1, k - 1)));
          dzeta[c] = 0.25 * ((P_(c, i, j, k) + P_(c, i, j - 1, k) + P_(c, i - 1, j, k) + P_(c, i - 1, j - 1, k)) -
                             (P_(c, i, j, k - 1) + P_(c, i, j - 1, k - 1) + P_(c, i - 1, j, k - 1) + P_(c, i - 1, j - 1, k - 1)));
        }
        const double J = dxi[0] * (deta[1] * dzeta[2] - deta[2] * dzeta[1]) -
                         dxi[1] * (deta[0] * dzeta[2] - deta[2] * dzeta[0]) +
                         dxi[2] * (deta[0] * dzeta[1] - deta[1] * dzeta[0]);
        if (fabs(J) < 1.0e-12) return O_ERR_FLOP_COUNT;
        aj[o_nidx(g, i, j, k)] = 1.0 / J;
      }
#undef P_
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t j = 0; j < my; ++j)
      if (1 < mx) aj[o_nidx(g, 0, j, k)] = aj[o_nidx(g, 1, j, k)];
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t j = 0; j < my; ++j)
      if (mx - 2 >= 0) aj[o_nidx(g, mx - 1, j, k)] = aj[o_nidx(g, mx - 2, j, k)];
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t i = 0; i < mx; ++i)
      if (1 < my) aj[o_nidx(g, i, 0, k)] = aj[o_nidx(g, i, 1, k)];
  for (int64_t k = 0; k < mz; ++k)
    for (int64_t i = 0; i < mx; ++i)
      if (my - 2 >= 0) aj[o_nidx(g, i, my - 1, k)] = aj[o_nidx(g, i, my - 2, k)];
  for (int64_t j = 0; j < my; ++j)
    for (int64_t i = 0; i < mx; ++i)
      if (1 < mz) aj[o_nidx(g, i, j, 0)] = aj[o_nidx(g, i, j, 1)];
  for (int64_t j = 0; j < my; ++j)
    for (int64_t i = 0; i < mx; ++i)
      if (mz - 2 >= 0) aj[o_nidx(g, i, j, mz - 1)] = aj[o_nidx(g, i, j, mz - 2)];
  return 0;
}

/* Metric.c:195-260 (VecMin / VecMax over every node). */
int o_CheckAndFixGridOrientation(const OGrid *g, double *csi, double *eta, double *zet, double *aj,
                                 int *flipped) {
  const int64_t nn = (g->IM + 1) * (g->JM + 1) * (g->KM + 1);
  double lo = aj[0], hi = aj[0];
  for (int64_t q = 1; q < nn; ++q) {
    if (aj[q] < lo) lo = aj[q];
    if (aj[q] > hi) hi = aj[q];
  }
  if (flipped) *flipped = 0;
  if (lo < 0.0 && hi > 0.0) return O_ERR_USER;
  if (hi < 0.0) {
    for (int64_t q = 0; q < 3 * nn; ++q) { csi[q] = -csi[q]; eta[q] = -eta[q]; zet[q] = -zet[q]; }
    for (int64_t q = 0; q < nn; ++q) aj[q] = -aj[q];
    if (flipped) *flipped = 1;
  }
  return 0;
}

/* setup.c:1294-1420, one rank: cells 1 .. IM-1 (x), 1 .. JM-1 (y), 1 .. KM-1 (z). */
int o_Contra2Cart(const OGrid *g, const double *ucont, const double *csi, const double *eta,
                  const double *zet, double *ucat) {
  for (int64_t k = 1; k < g->KM; ++k)
    for (int64_t j = 1; j < g->JM; ++j)
      for (int64_t i = 1; i < g->IM; ++i) {
        const int64_t n = o_nidx(g, i, j, k);
        const int64_t ni = o_nidx(g, i - 1, j, k), nj = o_nidx(g, i, j - 1, k), nk = o_nidx(g, i, j, k - 1);
        double m[3][3];
        for (int c = 0; c < 3; ++c) {
          m[0][c] = 0.5 * (csi[3 * ni + c] + csi[3 * n + c]);
          m[1][c] = 0.5 * (eta[3 * nj + c] + eta[3 * n + c]);
          m[2][c] = 0.5 * (zet[3 * nk + c] + zet[3 * n + c]);
        }
        double q[3];
        q[0] = 0.5 * (ucont[3 * ni] + ucont[3 * n]);
        q[1] = 0.5 * (ucont[3 * nj + 1] + ucont[3 * n + 1]);
        q[2] = 0.5 * (ucont[3 * nk + 2] + ucont[3 * n + 2]);
        const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                           m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        if (fabs(det) < 1.0e-18) return O_ERR_FLOP_COUNT;
        const double det_inv = 1.0 / det;
        const double det0 = q[0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                            q[1] * (m[0][1] * m[2][2] - m[0][2] * m[2][1]) +
                            q[2] * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
        const double det1 = -q[0] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                            q[1] * (m[0][0] * m[2][2] - m[0][2] * m[2][0]) -
                            q[2] * (m[0][0] * m[1][2] - m[0][2] * m[1][0]);
        const double det2 = q[0] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]) -
                            q[1] * (m[0][0] * m[2][1] - m[0][1] * m[2][0]) +
                            q[2] * (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
        ucat[3 * n] = det0 * det_inv;
        ucat[3 * n + 1] = det1 * det_inv;
        ucat[3 * n + 2] = det2 * det_inv;
      }
  return 0;
}
