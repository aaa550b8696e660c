/*
 * fdf_gb300.h -- C ABI of the GB300-native particle hot path of PICurv
 * (VishalKandala/fdf): walking-search cell location, trilinear interpolation of
 * cell-centred ucat, explicit position update, and particle-to-grid deposits.
 *
 * The reference's hot path is a set of C functions on PETSc objects
 * (UserCtx, DMSwarm, DMDA Vec) returning PetscErrorCode.  This library keeps
 * their names, argument meaning and error behaviour, with the PETSc objects
 * replaced by an opaque FdfContext that holds the grid and the swarm
 * device-resident on one GPU (one rank owning the whole domain: no migration).
 *
 *   - Plain pointers and sizes only; host pointers are ordinary (or pinned)
 *     host memory, laid out exactly as the reference's DMSwarm / DMDA arrays.
 *   - Every function returns 0 or a PETSc error code (same numbering as
 *     petscerror.h).  A particle that cannot be located is not an error: its
 *     status becomes LOST and its cell (-1,-1,-1), as in the reference.
 *   - PetscInt is 64-bit in the reference's own build (PETSc 3.19.2-64bit), so
 *     cell indices and statuses cross this boundary as int64_t.
 *   - Calls on one context are issued on that context's CUDA stream and return
 *     once the work is queued; functions that return host data synchronise.
 */
#ifndef FDF_GB300_H
#define FDF_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes (PETSc numbering). */
#define FDF_SUCCESS 0
#define FDF_ERR_MEM 55
#define FDF_ERR_SUP 56
#define FDF_ERR_ARG_WRONG 62
#define FDF_ERR_ARG_OUTOFRANGE 63
#define FDF_ERR_ARG_WRONGSTATE 73
#define FDF_ERR_LIB 76
#define FDF_ERR_USER 83          /* degenerate cell face met by the walk (walkingsearch.c:147-155) */
#define FDF_ERR_FLOP_COUNT 90    /* near-zero Jacobian or Contra2Cart determinant (Metric.c:560, setup.c:1389) */
#define FDF_ERR_ARG_NULL 85
#define FDF_ERR_GPU 97

/* ParticleLocationStatus (common.h:75-124). */
#define FDF_NEEDS_LOCATION 0
#define FDF_ACTIVE_AND_LOCATED 1
#define FDF_MIGRATING_OUT 2
#define FDF_LOST 3
#define FDF_UNINITIALIZED 4

/* BoundingBox (common.h:145-148). */
typedef struct { double min_coords[3]; double max_coords[3]; } FdfBoundingBox;

typedef struct FdfContext FdfContext;

/* Per-step bookkeeping that the reference reports through its removal calls. */
typedef struct {
  int64_t n_start;         /* live particles when the step began            */
  int64_t n_end;           /* live particles after removal                  */
  int64_t removed_lost;    /* CheckAndRemoveLostParticles count             */
  int64_t removed_oob;     /* CheckAndRemoveOutOfBoundsParticles count      */
  int64_t walk_evals;      /* cell evaluations the reference's walk makes (a walk that cycles
                              until MAX_TRAVERSAL counts 1000; the GPU walk stops at the cycle) */
  int64_t fp64_fallbacks;  /* walk faces whose class needed the exact FP64 distance (every form) */
} FdfStepInfo;

/* Forms of the path.  PLAIN_FP64: every value as the reference computes it, bit for bit.
 * FP32: interpolation, advection and deposition in FP32 (compensated deposit sums),
 * positions kept in FP64, and every walk decision -- hence every cell and status --
 * exactly the FP64 reference's for the form's own positions (FP32 signed distances
 * with a rigorous error bound, exact FP64 distance where the bound cannot decide). */
#define FDF_FORM_PLAIN_FP64 0
#define FDF_FORM_FP32 1
/* LEARNED_FP32: the FP32 form with a trained network (fdf_Locator*) in its walk.  After the
 * reference's first evaluation (in the previous cell), a particle estimated at least two cells
 * away (fdf_LocatorSetMinDistance) gets a predicted cell from the network, and the reference
 * walk continues from its second cell P1 with the plane-table rows of the path from P1 toward
 * the predicted cell fetched ahead of its evaluations.  The walk itself is the reference's, so
 * cells, weights and statuses are the FP32 form's for every input, whatever the network
 * predicts: a walk that started at the prediction could end elsewhere, because the reference
 * accepts any cell whose extended face plane passes within 1e-11 h of the point
 * (walkingsearch.c:427-459), and which such cell it meets depends on its path. */
#define FDF_FORM_LEARNED_FP32 2

/* ---- context, grid and fields (replace UserCtx set-up: setup.c:197-290, grid.c:34-160) ---- */
int fdf_ContextCreate(FdfContext **ctx, int device);
int fdf_ContextDestroy(FdfContext *ctx);
/* Node coordinates, DMDA coordinate layout [KM+1][JM+1][IM+1][3] (grid.c:356-383).
 * Builds the per-cell face-plane table and the bounding box (grid.c:762-883). */
int fdf_SetGrid(FdfContext *ctx, int64_t IM, int64_t JM, int64_t KM, const double *coor);
/* Cell-centred Cartesian velocity.  node_sized=1: the reference's DMDA layout
 * [KM+1][JM+1][IM+1][3] with cell (i,j,k) at [k][j][i]; node_sized=0: [KM][JM][IM][3]. */
int fdf_SetUcat(FdfContext *ctx, const double *ucat, int node_sized);
/* Reads the context's cell-centred ucat back, in either layout of fdf_SetUcat (node_sized=1:
 * the extra i=IM, j=JM, k=KM entries are zero). */
int fdf_GetUcat(FdfContext *ctx, double *ucat, int node_sized);

/* ---- Eulerian input: contravariant face velocity -> ucat, on the device ---- */
/* Face metrics Csi, Eta, Zet (ComputeFaceMetrics, Metric.c:286-460) and Aj = 1/J
 * (ComputeCellCenteredJacobianInverse, Metric.c:491-600) of the grid, after the orientation
 * check (CheckAndFixGridOrientation, Metric.c:195-260), node-sized [KM+1][JM+1][IM+1][3]
 * (aj: [KM+1][JM+1][IM+1]); any output may be NULL.  *flipped = 1 when every Aj was negative
 * and all four were negated (the reference's GridOrientation is +1 afterwards either way).
 * Errors: FDF_ERR_FLOP_COUNT (|J| < 1e-12 at a node), FDF_ERR_USER (Aj of mixed signs). */
int fdf_GetGridMetrics(FdfContext *ctx, double *csi, double *eta, double *zet, double *aj, int *flipped);
/* Contravariant face velocity, the reference's lUcont: node-sized [KM+1][JM+1][IM+1][3] with
 * .x the flux through i-face i, .y through j-face j, .z through k-face k at node (i,j,k). */
int fdf_SetUcont(FdfContext *ctx, const double *ucont);
/* Contra2Cart(UserCtx*) (setup.c:1294-1420): ucat of the cells i in 1..IM-1, j in 1..JM-1,
 * k in 1..KM-1 (the reference's interior loop on one rank) from the face velocity and the
 * orientation-fixed metrics, bit-identical to the reference; the other cells keep their
 * ucat (the reference leaves them to its boundary conditions).  The metrics and the grid-only
 * part of Cramer's rule are built on the first call for a grid.  Stream-ordered: the next
 * step, fdf_GetUcat and fdf_Synchronize see the result.  Errors: FDF_ERR_ARG_WRONGSTATE
 * without fdf_SetUcont, the errors of fdf_GetGridMetrics, FDF_ERR_FLOP_COUNT (a cell's
 * |det| < 1e-18; ucat is then left unchanged). */
int fdf_Contra2Cart(FdfContext *ctx);
/* Contra2Cart from a face velocity already in device memory (a solver that keeps lUcont on the
 * GPU): ucont_device, node-sized [KM+1][JM+1][IM+1][3] on the context's device, is read in place,
 * without a copy, on the context stream (fdf_GetStream): the caller orders its writes of the
 * array before the call.  FDF_ERR_ARG_WRONG when the pointer is not memory of that device. */
int fdf_Contra2CartDevice(FdfContext *ctx, const double *ucont_device);

/* Selects the form used by the next fdf_SetSwarm (default PLAIN_FP64). */
int fdf_SetForm(FdfContext *ctx, int form);
int fdf_SetTimeStep(FdfContext *ctx, double dt);                 /* user->dt            */
int fdf_SetParticleVolume(FdfContext *ctx, double volume);       /* face deposit V_p    */

/* ---- swarm transfer (DMSwarm fields, ParticleSwarm.c:64-96, [n][bs] layout) ----
 * Route (fdf_SetTransferRoute): STAGED copies the arrays with the copy engines, in particle
 * chunks, through a device staging buffer, the layout conversion of one chunk overlapping the
 * copies of the next; IN_PLACE has the layout kernels read (fdf_SetSwarm) or write
 * (fdf_GetSwarm) the arrays over the host link when all seven arrays of a call are page-locked
 * host memory (cudaHostAlloc / cudaHostRegister) and 16-byte aligned, and falls back to STAGED
 * otherwise.  Which is faster depends on the machine (on the GB300s tried, the copy engines ran
 * at the link's rate on one and kernel accesses at a quarter of it; on two others the in-place
 * route was 19-39 % faster).  AUTO (default), per direction: the first call with page-locked
 * arrays and at least 4M particles moves two slices of its particles (up to 4M each) by each
 * route, timed with events, and that call's remaining particles and every later call of that
 * direction take the faster route; smaller calls and other arrays go STAGED.  The results are
 * the same by either route.  fdf_GetTransferRoutes reports the routes chosen (-1: AUTO has not
 * measured that direction yet); fdf_SetTransferRoute(AUTO) measures again. */
#define FDF_TRANSFER_STAGED 0
#define FDF_TRANSFER_IN_PLACE 1
#define FDF_TRANSFER_AUTO 2
int fdf_SetTransferRoute(FdfContext *ctx, int route);
int fdf_GetTransferRoutes(FdfContext *ctx, int *upload, int *download);
int fdf_ReserveParticles(FdfContext *ctx, int64_t capacity);
int fdf_SetSwarm(FdfContext *ctx, int64_t n, const double *position, const double *velocity,
                 const double *weight, const double *P, const int64_t *cell_id, const int64_t *pid,
                 const int64_t *status);
/* Replaces the swarm by n particles seeded on the device like the reference's volumetric
 * initialisation (ParticleSwarm.c:229-312 + Metric.c:48-62): a random cell and random
 * logical coordinates from counter-based splitmix64 streams (seed), bit-identical to the
 * harness generator fdf_gb300/workloads.py volumetric_particles.  PIDs pid_base + p, P as
 * given, status UNINITIALIZED; DMSwarm_CellID is the generating cell when
 * start_in_generating_cell, else (-1,-1,-1) (the reference's corner start). */
int fdf_SeedParticles(FdfContext *ctx, int64_t n, uint64_t seed, int start_in_generating_cell, int64_t pid_base,
                      double P);
int fdf_GetSwarmSize(FdfContext *ctx, int64_t *n);
int fdf_GetSwarm(FdfContext *ctx, int64_t n_max, int64_t *n, double *position, double *velocity,
                 double *weight, double *P, int64_t *cell_id, int64_t *pid, int64_t *status);

/* ---- Eulerian outputs ---- */
/* ParticleCount and the P average, node-sized [KM+1][JM+1][IM+1] (interpolation.c:2063-2116). */
int fdf_GetScatteredFields(FdfContext *ctx, double *count, double *P_avg);
/* Corner (node) velocity that the interpolation averages from ucat (interpolation.c:598-679),
 * every node, [KM+1][JM+1][IM+1][3]. */
int fdf_GetCornerField(FdfContext *ctx, double *corner);
/* Face volume deposits: fi [KM][JM][IM+1], fj [KM][JM+1][IM], fk [KM+1][JM][IM].
 * No counterpart in the reference (its only deposit is the cell average of P):
 * a particle of volume V in cell (i,j,k) with weights (a1,a2,a3) gives (1-a)V/3
 * to the lower and aV/3 to the upper face of each logical direction. */
int fdf_GetFaceDeposits(FdfContext *ctx, double *fi, double *fj, double *fk);
/* Momentum face deposit (no counterpart in the reference): when enabled, every step also
 * deposits V * velocity (the velocity interpolated in that step) with the volume's split,
 * summed in the same order.  Outputs [faces][3]: mi [KM][JM][IM+1][3], mj [KM][JM+1][IM][3],
 * mk [KM+1][JM][IM][3].  Enabling allocates 36 B per face (FP64 + FP32 copies). */
int fdf_SetMomentumDeposit(FdfContext *ctx, int enable);
int fdf_GetFaceMomentum(FdfContext *ctx, double *mi, double *mj, double *mk);

/* ---- the hot path ---- */
/* PerformInitialSetup_TEST (simulation.c:129-175): locate every particle, interpolate,
 * scatter and deposit.  LOST particles are kept (the reference removes them in step 1). */
int fdf_PerformInitialSetup(FdfContext *ctx, FdfStepInfo *info);
/* One step of AdvanceSimulation_TEST (simulation.c:240-297): ResetAllParticleStatuses,
 * UpdateAllParticlePositions, LocateAllParticlesInGrid_TEST, CheckAndRemoveLostParticles,
 * CheckAndRemoveOutOfBoundsParticles, InterpolateAllFieldsToSwarm,
 * ScatterAllParticleFieldsToEulerFields, plus the face deposit; the particles are
 * re-sorted by cell.  info may be NULL (then nothing is read back and the call does
 * not synchronise). */
int fdf_AdvanceStep(FdfContext *ctx, FdfStepInfo *info);
int fdf_AdvanceSteps(FdfContext *ctx, int nsteps);

/* ---- the same stages one call at a time, for callers that keep the reference's loop ----
 * Called in the reference's order (reset, update, locate, remove LOST, remove out of bounds,
 * interpolate, scatter) they give bit for bit what fdf_AdvanceStep gives. */
/* ResetAllParticleStatuses (ParticleMotion.c:2149-2176): ACTIVE_AND_LOCATED -> NEEDS_LOCATION. */
int fdf_ResetAllParticleStatuses(FdfContext *ctx);
/* UpdateAllParticlePositions (ParticleMotion.c:38-95): position += velocity * dt. */
int fdf_UpdateAllParticlePositions(FdfContext *ctx);
/* LocateAllParticlesInGrid_TEST (ParticleMotion.c:1931-2135): the walk for every particle not
 * ACTIVE_AND_LOCATED, from its previous cell; LOST particles are kept (at the end of the
 * cell-sorted order).  Velocities are not touched. */
int fdf_LocateAllParticlesInGrid(FdfContext *ctx, FdfStepInfo *info);
/* CheckAndRemoveLostParticles (ParticleMotion.c:532-625); *removed (optional) = count. */
int fdf_CheckAndRemoveLostParticles(FdfContext *ctx, int64_t *removed);
/* CheckAndRemoveOutOfBoundsParticles (ParticleMotion.c:283-383): positions outside the
 * grid's bounding box widened by 1e-6 (grid.c:816-858); *removed (optional) = count. */
int fdf_CheckAndRemoveOutOfBoundsParticles(FdfContext *ctx, int64_t *removed);
/* InterpolateAllFieldsToSwarm (interpolation.c:1660-1711): center->corner and the trilinear
 * velocity of every particle from its cell and weights; statuses are kept. */
int fdf_InterpolateAllFieldsToSwarm(FdfContext *ctx);
/* ScatterAllParticleFieldsToEulerFields (interpolation.c:2223-2313): ParticleCount and the P
 * average, plus the face deposit (read them with fdf_GetScatteredFields, fdf_GetFaceDeposits). */
int fdf_ScatterAllParticleFieldsToEulerFields(FdfContext *ctx);

/* LocateParticleOrFindMigrationTarget_TEST (walkingsearch.c:1094-1242) for a batch of points
 * that are not the swarm (probes, post-processing): the plain FP64 walk, bit-identical to the
 * reference, from cell_in[p] (or cell (0,0,0), a new particle's start, where it is -1 or
 * cell_in is NULL).  Outputs: cell_out [n][3] (-1 when LOST), weight [n][3] (zero when LOST),
 * status [n] (ACTIVE_AND_LOCATED or LOST).  Host arrays; the swarm is not touched. */
int fdf_LocatePoints(FdfContext *ctx, int64_t n, const double *position, const int64_t *cell_in, int64_t *cell_out,
                     double *weight, int64_t *status);

/* InterpolateEulerFieldToSwarm (interpolation.c:1205-1399) for particles the caller holds (a
 * DMSwarm kept on the host, probes): the velocity of n particles from their cells cell [n][3] and
 * weights weight [n][3], in the caller's order, bit-identical to the reference; a cell index
 * outside 0..IM-1, 0..JM-1, 0..KM-1 gives velocity zero, as the reference's stencil guard does.
 * The corner field is made from the context's ucat (every node).  Host arrays. */
int fdf_InterpolatePoints(FdfContext *ctx, int64_t n, const int64_t *cell, const double *weight, double *velocity);

/* ---- k-slab decomposition over several GPUs (fdf_gb300/slabs.py drives these) ----
 * The reference distributes particles over MPI ranks with DMSwarmMigrate
 * (ParticleMotion.c:1931-2135, the walk-and-handoff passes).  Here each rank holds the whole grid
 * and the particles whose cell lies in its k-slab of cells; after the walk the particles that
 * left the slab move to their slab's rank, and the k-faces between two slabs are summed by the
 * upper rank from the lower rank's partial sums, so the ranks' results together are the one-rank
 * results bit for bit (plain form). */
/* The held particles whose cell has k outside [k_lo, k_hi) leave the context into the host arrays
 * (DMSwarm layout, in the held order -- by cell, within a cell by PID in the plain form: cells
 * below the slab, then above); particles without a cell stay.  *n = the number extracted
 * (FDF_ERR_ARG_OUTOFRANGE, nothing moved, if > n_max). */
int fdf_ExtractParticles(FdfContext *ctx, int64_t k_lo, int64_t k_hi, int64_t n_max, int64_t *n, double *position,
                         double *velocity, double *weight, double *P, int64_t *cell_id, int64_t *pid, int64_t *status);
/* Particles from another rank join the held swarm with their cells, weights and statuses (the
 * capacity reserved before fdf_SetSwarm must hold them). */
int fdf_AddParticles(FdfContext *ctx, int64_t n, const double *position, const double *velocity, const double *weight,
                     const double *P, const int64_t *cell_id, const int64_t *pid, const int64_t *status);
/* The plain form's k-faces of layer k (between cells k-1 and k) after a deposit, summed again as
 * seed[j][i] (the lower cell's part, made by the rank holding it: that rank's own values of this
 * layer) followed by the held particles of cells (i, j, k), in the deposit's order; momentum seeds
 * [j][i][3] (NULL: zero) when the momentum deposit is on.  FDF_ERR_SUP in the precision forms. */
int fdf_DepositKFaceLayer(FdfContext *ctx, int64_t k, const double *seed, const double *seed_momentum);

/* ---- sort by cell (the per-step re-sort of the hot path, as a standalone call) ---- */
/* Stable counting sort of n particle slots by cell id, all pointers on the device.
 * Slots whose id is negative or >= ncells get no place.  On return cell_start[c] is the
 * first sorted slot of cell c (cell_start[ncells] = number of placed slots) and
 * perm[cell_start[c] .. cell_start[c+1]) lists cell c's slot indices in ascending
 * order.  Scratch is stream-ordered (cudaMallocAsync/cudaFreeAsync on `stream`).
 * No counterpart call in the reference, which keeps DMSwarm in insertion order; it
 * is the sort-by-cell step that makes the gathers of this library coalesced. */
int fdf_SortByCell(const int32_t *cell_ids, int64_t n, int64_t ncells, uint32_t *perm, uint32_t *cell_start,
                   void *stream);

/* fdf_SortByCell for callers that cannot allocate device memory (e.g. a host code whose
 * device memory is owned by another allocator, or a loop that must not enter one).
 * No counterpart in the reference.  Same arguments, results and ordering as
 * fdf_SortByCell; its scratch is a file-scope device array of ~4 MiB that every GPU
 * loading this library keeps until exit, so ncells is limited to FDF_NOALLOC_MAX_CELLS
 * (larger requests return FDF_ERR_ARG_OUTOFRANGE).  The first call on a device looks up
 * that array's address on the current device: make it outside stream capture.  All
 * calls share the array (each clears what must start at zero), so calls that overlap
 * on the GPU race: serialise them.  The looked-up address belongs to the device's primary
 * context: after a cudaDeviceReset of that device, do not call it again in the process.
 * Calls no cudaMalloc/cudaFree. */
#define FDF_NOALLOC_MAX_CELLS 1048576
int fdf_SortByCellNoAlloc(const int32_t *cell_ids, int64_t n, int64_t ncells, uint32_t *perm, uint32_t *cell_start,
                          void *stream);

/* ---- learned start-cell locator (FDF_FORM_LEARNED_FP32) ----
 * No counterpart in the reference, which starts each walk in the particle's previous cell
 * (walkingsearch.c:571-626).  A 3-128-128-128-3 SiLU network maps the normalised position
 * xhat = (x - centre) * inv_half (centre and half-extent of the grid's bounding box) to
 * y, read as cell index floor((y_d + 1) N_d / 2), N = (IM, JM, KM), clamped to the grid.
 * Weights are bfloat16 in every training product and, by default, in inference (FP32
 * accumulation in both; fdf_LocatorSetInferenceType), with FP32 master copies for training.
 * Parameters, one float vector of FDF_LOCATOR_NPARAM values:
 * W1 [128][3], b1 [128], W2 [128][128], b2, W3 [128][128], b3, W4 [3][128], b4 [3]. */
#define FDF_LOCATOR_NPARAM 33923
/* Weights uniform in +-1/sqrt(fan_in) from the seed, biases zero; Adam state cleared. */
int fdf_LocatorInit(FdfContext *ctx, uint64_t seed);
/* Trains on the device: n_samples points seeded like fdf_SeedParticles (seed), each located
 * by the plain FP64 walk from its generating cell; the located (position, cell) pairs are
 * the training set.  `steps` Adam steps on minibatches of `batch` pairs, learning rate lr
 * on a cosine schedule; loss = mean over the batch of sum_d (N_d/2 (y_d - t_d))^2 / 3 with
 * t_d = 2 (idx_d + 0.5) / N_d - 1 (squared error in cells).  loss_history (optional,
 * [steps]) receives the loss of every step.  Initialises the weights first if none are set. */
int fdf_LocatorTrain(FdfContext *ctx, int64_t n_samples, uint64_t seed, int64_t steps, int64_t batch, double lr,
                     float *loss_history);
int fdf_LocatorSetParams(FdfContext *ctx, const float *params, int64_t n);
int fdf_LocatorGetParams(FdfContext *ctx, float *params, int64_t n);
int fdf_LocatorGetNormalization(FdfContext *ctx, float *centre, float *inv_half);
/* Loss and gradients of the current weights on one batch given on the host: xhat [batch][3]
 * (already normalised), target [batch][3]; grads [FDF_LOCATOR_NPARAM]. */
int fdf_LocatorGradients(FdfContext *ctx, const float *xhat, const float *target, int64_t batch, float *grads,
                         float *loss);
/* Predicted cells (i, j, k) of n host positions [n][3]; outputs (optional) [n][3] = y. */
int fdf_LocatorPredict(FdfContext *ctx, const double *position, int64_t n, int64_t *cell_id, float *outputs);
/* Operand type of inference on the tensor cores: FDF_LOCATOR_BF16 (default; each normalised
 * coordinate enters as a bfloat16 pair hi + lo) or FDF_LOCATOR_F16 (half precision).  Only the
 * predictions, never the cells, depend on it. */
#define FDF_LOCATOR_BF16 0
#define FDF_LOCATOR_F16 1
int fdf_LocatorSetInferenceType(FdfContext *ctx, int type);
/* Which particles the learned form asks the network: after the reference's first evaluation
 * (in the previous cell), a particle estimated at least `cells` cells past that cell (from the
 * evaluation's face distances) gets a prediction and is walked from P1 in a second pass; a
 * nearer one continues the reference walk at once.  Default 2.0; 0 asks for every particle
 * that left its cell.  Results do not depend on it. */
int fdf_LocatorSetMinDistance(FdfContext *ctx, double cells);
/* Running totals of the learned form: particles given a prediction (asked); evaluations of their
 * walks from P1 whose cell lay on the predicted path, i.e. whose row was fetched ahead (on_path);
 * evaluations of those walks (walk_evals); and zero (unused). */
int fdf_LocatorGetStats(FdfContext *ctx, int64_t *asked, int64_t *on_path, int64_t *walk_evals, int64_t *unused);

/* ---- the reference's on-disk formats (host-side; no GPU work except the swarm transfers) ----
 * FDFGRID grid file (io.c:101-170 ReadGridFile, grid.c:356-383 AssignGridCoordinates): an
 * optional "FDFGRID" line, the number of blocks, "IM JM KM" (cells) per block, then one "x y z"
 * line per node, i fastest, then j, then k.  The first block is read; coor == NULL returns the
 * sizes only; coor_len counts doubles.  The writer emits one block with 17 significant digits. */
int fdf_ReadGridFile(const char *path, int64_t *IM, int64_t *JM, int64_t *KM, double *coor, int64_t coor_len);
int fdf_WriteGridFile(const char *path, int64_t IM, int64_t JM, int64_t KM, const double *coor);
/* PETSc binary Vec file as VecView writes it on one rank (WriteFieldData, io.c:653-700):
 * big-endian {VEC_FILE_CLASSID 1211214, N} as PetscInt (8 bytes when int64_indices, as in the
 * reference's PETSc 3.19.2-64bit build), then N big-endian doubles; bs > 1 also writes
 * "<path>.info" with "-vecload_block_size <bs>".  values == NULL reads the length only. */
int fdf_WritePetscVec(const char *path, const double *values, int64_t n, int bs, int int64_indices);
int fdf_ReadPetscVec(const char *path, double *values, int64_t n_max, int64_t *n, int int64_indices);
/* A real swarm field ("position", "velocity", "weight", "P") of the context written to, or read
 * from, such a file: WriteSwarmField (io.c:1023-1070) and ReadSwarmField (io.c:1924-1950) of the
 * reference, whose files are results/<field><step %05d>_0.dat.  Reading needs a swarm of the
 * file's length and replaces that field (the particles keep the swarm's current order). */
int fdf_WriteSwarmField(FdfContext *ctx, const char *field, const char *path, int int64_indices);
int fdf_ReadSwarmField(FdfContext *ctx, const char *field, const char *path, int int64_indices);

/* ---- utilities ---- */
int fdf_Synchronize(FdfContext *ctx);
/* The context's cudaStream_t, for callers that time or order work around it. */
void *fdf_GetStream(FdfContext *ctx);
const char *fdf_GetLastError(FdfContext *ctx);
/* Number of kernel launches the library has issued on this context. */
int64_t fdf_GetLaunchCount(FdfContext *ctx);
/* Stage timing with CUDA events on the context stream (enable resets the record).
 * Stages: 0 center->corner (on a second stream, concurrent with 2), 1 advect+locate,
 * 2 sort by cell (histogram scan, slots, per-cell PID order), 3 wait for stage 0,
 * 4 gather+interpolate, 5 deposits; learned form: 6 network inference, 7 walk from the
 * guess (its stage 1 is the first evaluation and the pending list); 8 fdf_Contra2Cart
 * (outside the steps, one span per call).  ms_total[s] sums the
 * stage over all pipeline runs since enabling; launches[s] counts the timed spans. */
int fdf_SetProfiling(FdfContext *ctx, int enable);
/* Running totals since fdf_SetSwarm: particles advanced (sum over steps of the live
 * particles at step start), walking-search cell evaluations actually made, and
 * corner nodes computed (the steps compute only nodes next to occupied cells). */
int fdf_GetCounters(FdfContext *ctx, int64_t *particle_steps, int64_t *walk_evals, int64_t *corner_nodes);
int fdf_GetStageTimes(FdfContext *ctx, double *ms_total, int64_t *launches, int nstages);

/* ---- testing ---- */
/* Failure injection on the host, for tests of the error paths (no counterpart in the
 * reference): the next `after` device allocations of the contexts' buffers succeed and every
 * later one fails as out of memory (FDF_ERR_MEM), until called again with a negative value
 * (no limit).  A context whose fdf_SetGrid or fdf_ReserveParticles failed this way holds no
 * grid (or no swarm) and returns FDF_ERR_ARG_WRONGSTATE from the calls that need one.
 * Process-wide; not for production use. */
int fdf_TestFailDeviceAllocations(int64_t after);
/* Time-out path of the learned locator's tensor-core kernel: fdf_LocatorPredict's launch on n
 * positions [n][3] with no MMA issued, so that each CTA's first bounded mbarrier wait (1024
 * polls) runs out; the CTAs free their tensor memory and return, and the call returns
 * FDF_ERR_GPU as a real time-out would.  Nothing is left in flight: the next call works.
 * No counterpart in the reference. */
int fdf_TestLocatorWaitTimeout(FdfContext *ctx, const double *position, int64_t n);
/* Time-out path of the locator's fused training kernel: fdf_LocatorGradients' training launch on
 * the batch xhat, target [batch][3] with no MMA issued, so that each CTA's first bounded mbarrier
 * wait (1024 polls) runs out; the CTAs free their tensor memory and return, and the call returns
 * FDF_ERR_GPU as a real time-out would.  Nothing is left in flight and the weights are untouched:
 * the next call works.  No counterpart in the reference. */
int fdf_TestLocatorTrainTimeout(FdfContext *ctx, const float *xhat, const float *target, int64_t batch);

#ifdef __cplusplus
}
#endif
#endif
