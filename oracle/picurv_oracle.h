/*
 * picurv_oracle.h -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
 *
 * CPU restatement of PICurv's Lagrangian particle hot path (VishalKandala/fdf),
 * used only as the checker for the CUDA implementation in fdf_gb300/ (by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py).
 *
 * Every function follows one reference function literally: same operation order,
 * no FMA contraction (built with -ffp-contract=off), same constants, same quirks.
 * Each definition cites the reference file:line it restates.
 *
 * Parity status: the reference ships no test vectors for this path (its only
 * test-like file, old/test_walkingsearch.c, does not compile against the live
 * code), so this restatement is pinned by known-answer tests derived from the
 * reference's logic (tests/test_oracle_kats.py) -- parity unpinned at the
 * reference level.
 */
#ifndef PICURV_ORACLE_H
#define PICURV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double x, y, z; } OCmpnts;          /* common.h:46-48 Cmpnts        */
typedef struct { OCmpnts vertices[8]; } OCell;       /* common.h:153-155 Cell        */

enum { O_LEFT = 0, O_RIGHT, O_BOTTOM, O_TOP, O_FRONT, O_BACK, O_NUM_FACES };  /* common.h:129-137 */
enum { O_NEEDS_LOCATION = 0, O_ACTIVE_AND_LOCATED = 1, O_MIGRATING_OUT = 2,
       O_LOST = 3, O_UNINITIALIZED = 4 };                                     /* common.h:75-124 */

/* PETSc error codes the path can raise (same numbering as petscerror.h). */
#define O_ERR_ARG_NULL 85
#define O_ERR_USER 83

/* A one-rank DMDA grid: node coordinates [KM+1][JM+1][IM+1][3], i fastest. */
typedef struct {
  int64_t IM, JM, KM;
  const double *coor;
} OGrid;

/* DMSwarm fields of one rank (ParticleSwarm.c:64-96), [n][bs] arrays.
 * Removal shrinks n in place with DMSwarm's swap-with-last semantics. */
typedef struct {
  int64_t n;
  double *pos;      /* position [n][3]                 */
  double *vel;      /* velocity [n][3]                 */
  double *weight;   /* weight   [n][3]                 */
  double *P;        /* P        [n]                    */
  int64_t *cell;    /* DMSwarm_CellID [n][3] (64-bit PetscInt build) */
  int64_t *pid;     /* DMSwarm_pid [n]                 */
  int64_t *status;  /* DMSwarm_location_status [n]     */
} OSwarm;

/* ---- walkingsearch.c restatements ------------------------------------- */
int o_GetCellCharacteristicSize(const OCell *cell, double *cellSize);
int o_ComputeSignedDistanceToPlane(OCmpnts v1, OCmpnts v2, OCmpnts v3, OCmpnts v4,
                                   OCmpnts cell_centroid, OCmpnts p_target,
                                   double *d_signed, double threshold);
int o_CalculateDistancesToCellFaces(OCmpnts p, const OCell *cell, double *d, double threshold);
int o_DeterminePointPosition(const double *d, int64_t *result);
int o_GetCellVerticesFromGrid(const OGrid *g, int64_t idx, int64_t idy, int64_t idz, OCell *cell);
int o_EvaluateParticlePosition(const OCell *cell, double *d, OCmpnts p, int64_t *position, double threshold);
int o_UpdateCellIndicesBasedOnDistancesTEST(const double d[6], int64_t *idx, int64_t *idy, int64_t *idz);
int o_UpdateParticleWeights(double *d, double weights[3]);
/* One particle: cell[3], weights[3] in/out; status out; steps out = evaluations used. */
int o_LocateParticleOrFindMigrationTarget(const OGrid *g, const double loc[3], int64_t cell[3],
                                          double weights[3], int64_t *status, int64_t *steps);

/* ---- ParticleMotion.c / interpolation.c restatements ------------------- */
void o_ResetAllParticleStatuses(OSwarm *s);
void o_UpdateAllParticlePositions(OSwarm *s, double dt, int nthreads);
/* evals_out (optional): total walk evaluations. Returns 0 or O_ERR_USER (degenerate face). */
int o_LocateAllParticlesInGrid(const OGrid *g, OSwarm *s, int nthreads, int64_t *evals_out);
void o_CheckAndRemoveLostParticles(OSwarm *s, int64_t *removed);
void o_ComputeLocalBoundingBox(const OGrid *g, double bmin[3], double bmax[3]);
void o_CheckAndRemoveOutOfBoundsParticles(const OGrid *g, OSwarm *s, int64_t *removed);
/* ucat and corner are node-sized DMDA arrays [KM+1][JM+1][IM+1][3]; cell (i,j,k) at [k][j][i]. */
void o_InterpolateFieldFromCenterToCorner_Vector(const OGrid *g, const double *ucat, double *corner, int nthreads);
void o_TrilinearInterpolation_Vector(const OGrid *g, const double *corner, int64_t i, int64_t j, int64_t k,
                                     double a1, double a2, double a3, double out[3]);
void o_InterpolateEulerFieldToSwarm(const OGrid *g, const double *corner, OSwarm *s, int nthreads);
/* count, avg: node-sized [KM+1][JM+1][IM+1]. */
void o_ScatterParticleFieldToEulerField_P(const OGrid *g, const OSwarm *s, double *count, double *avg);

/* ---- Face deposit (defined by this build; no counterpart in the reference) ----
 * Particle volume V in cell (i,j,k) with weights (a1,a2,a3) adds (1-a)*(V/3) to the
 * lower face and a*(V/3) to the upper face of each logical direction.
 * fi: [KM][JM][IM+1], fj: [KM][JM+1][IM], fk: [KM+1][JM][IM].  abs_* (optional)
 * receive the sum of |contribution| per face, the scale for a tolerance.
 * mom_* (optional, [..][3]) receive the same split of V*velocity. */
void o_DepositParticlesToFaces(const OGrid *g, const OSwarm *s, double volume,
                               double *fi, double *fj, double *fk,
                               double *mom_i, double *mom_j, double *mom_k,
                               double *abs_i, double *abs_j, double *abs_k);

/* One full reference time step (simulation.c:240-311) on one rank:
 * reset -> advect -> locate -> remove LOST -> remove out-of-bounds -> center-to-corner
 * -> interpolate -> scatter P.  Deposit outputs are optional (NULL skips). */
typedef struct {
  int64_t removed_lost, removed_oob, evals, n_start;
} OStepInfo;
int o_AdvanceStep(const OGrid *g, const double *ucat, double *corner_scratch, OSwarm *s, double dt,
                  double *count, double *avg, int nthreads, OStepInfo *info);
/* PerformInitialSetup_TEST (simulation.c:129-175): locate -> interpolate -> scatter. */
int o_InitialSetup(const OGrid *g, const double *ucat, double *corner_scratch, OSwarm *s,
                   double *count, double *avg, int nthreads, OStepInfo *info);

/* ---- the Eulerian input of the path: metrics and Contra2Cart ------------ */
#define O_ERR_FLOP_COUNT 90
/* Metric.c:286-460 ComputeFaceMetrics: Csi, Eta, Zet at every node, node-sized
 * [KM+1][JM+1][IM+1][3]; outputs are zeroed first (fresh PETSc Vecs are zero). */
void o_ComputeFaceMetrics(const OGrid *g, double *csi, double *eta, double *zet);
/* Metric.c:491-600 ComputeCellCenteredJacobianInverse: Aj = 1/J, node-sized; returns
 * O_ERR_FLOP_COUNT at the first node with |J| < 1e-12. */
int o_ComputeCellCenteredJacobianInverse(const OGrid *g, double *aj);
/* Metric.c:195-260 CheckAndFixGridOrientation: Aj of mixed signs -> O_ERR_USER; all negative
 * -> Csi, Eta, Zet and Aj negated (*flipped = 1). */
int o_CheckAndFixGridOrientation(const OGrid *g, double *csi, double *eta, double *zet, double *aj,
                                 int *flipped);
/* setup.c:1294-1420 Contra2Cart: ucat (node-sized [..][3]) of the cells i in 1..IM-1,
 * j in 1..JM-1, k in 1..KM-1 from ucont (node-sized [..][3]) and the face metrics; other
 * entries are left alone.  Returns O_ERR_FLOP_COUNT at the first cell with |det| < 1e-18. */
int o_Contra2Cart(const OGrid *g, const double *ucont, const double *csi, const double *eta,
                  const double *zet, double *ucat);

#ifdef __cplusplus
}
#endif
#endif
