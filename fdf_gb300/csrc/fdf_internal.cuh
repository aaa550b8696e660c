// fdf_internal.cuh -- device-resident state and kernel declarations of the
// GB300 particle hot path (locate -> interpolate -> advect -> deposit).
//
// Data layout in HBM (one GPU holds the whole domain):
//   grid   : node coordinates, AoS [Nn][3] f64 (only used to build the plane table and bbox)
//            plane table, [Nc][FDF_ROW] f64: per cell, for each face f (LEFT..BACK)
//            the face centroid fc and the oriented unit normal n, then the cell's
//            distance threshold and a degenerate flag (304 B per cell)
//            ucat, SoA [3][Nc] f64 (cell-centred)
//            corner field, SoA [3][Nn] f64
//   swarm  : SoA, double-buffered so the per-step re-sort by cell is a gather
//            x y z u v w a1 a2 a3 P : f64 [cap]; pid : i64 [cap]; cell : i32 [cap]
//            (linear cell id i + IM*(j + JM*k), -1 = none); status : u8 [cap]
//   outputs: count, avg (node-sized [Nn] f64, the reference's ParticleCount / P);
//            face volume deposits fi [KM][JM][IM+1], fj [KM][JM+1][IM], fk [KM+1][JM][IM]
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#define FDF_ROW 38            // doubles per plane-table row (36 plane values + thr + flag)
#define FDF_ROW32 32          // floats per FP32 plane-table row: 128 B (c0 pair, thr32, slack, 6 x (n32, e32))
#define FDF_MAX_TRAVERSAL 1000
#define FDF_DISTANCE_THRESHOLD 1e-11
#define FDF_INTERP_DIST_TOL 1e-14
#define FDF_BBOX_TOL 1e-6
#define FDF_MAX_PARTICLES (512LL * 1024 * 1024)   // particle slots of one context or one sort call
#define FDF_PATH_LOOKAHEAD 2  // cells of the learned path whose table rows the walk from P1 prefetches

// Face order of the reference (common.h Face enum).
enum { F_LEFT = 0, F_RIGHT = 1, F_BOTTOM = 2, F_TOP = 3, F_FRONT = 4, F_BACK = 5 };
// Particle status values of the reference (common.h ParticleLocationStatus).
enum { ST_NEEDS_LOCATION = 0, ST_ACTIVE_AND_LOCATED = 1, ST_MIGRATING_OUT = 2, ST_LOST = 3,
       ST_UNINITIALIZED = 4 };

// Device error word bits.
enum { ERRBIT_DEGENERATE = 1u, ERRBIT_TC_TIMEOUT = 4u };

// The walk kernels' block flushes go to one of FDF_CNT_STRIPES rows (by block index), so that
// they spread over the L2 slices instead of queueing on one line; k_fold_counts adds the rows
// to the counters at the end of every pipeline run and zeroes them.
#define FDF_CNT_STRIPES 512
enum { CNT_LOST = 0, CNT_OOB = 1, CNT_EVALS = 2, CNT_EVALS_TOTAL = 3, CNT_LOST_TOTAL = 4, CNT_FB = 5,
       CNT_SLOTS = 8 };

// Counters kept on the device so that a step needs no host round trip.
struct DevCounters {
  // reset at the start of every pipeline run
  unsigned long long removed_lost;
  unsigned long long removed_oob;
  unsigned long long evals;        // walk evaluations the reference makes for this run (cycles count MAX_TRAVERSAL)
  unsigned long long lost_total;
  unsigned long long fallbacks;    // precision form: faces decided by the exact FP64 distance
  unsigned long long pending;      // learned form: particles that left their previous cell
  // kept across runs
  unsigned int err;
  unsigned int pad;
  int n;            // live particle count after the last removal
  int n_sorted;     // particles held in the arrays (live + LOST kept by the initial setup)
  unsigned long long psteps_total;  // sum over steps of the particles at step start (never reset per step)
  unsigned long long evals_total;   // walk evaluations actually made, all pipeline runs (never reset per step)
  unsigned long long nodes_total;   // corner nodes computed by the steps (never reset per step)
  unsigned long long fallbacks_total;
  unsigned long long guess_asked_total;   // learned form: particles given a guess (walked from P1)
  unsigned long long guess_taken_total;   // ... their walks' evaluations after P1 whose cell lay on the guessed path
  unsigned long long guess_evals_total;   // ... evaluations made by their walks from P1
  unsigned long long fallback_evals_total;   // (unused: zero)
  unsigned long long stripes[FDF_CNT_STRIPES][CNT_SLOTS];   // pending block flushes (k_fold_counts)
};
// The counters without the flush rows (what the host reads back).
#define DEVCOUNTERS_HEAD offsetof(DevCounters, stripes)

struct SwarmBuf {
  double *x, *y, *z;                         // positions (both forms)
  double *u, *v, *w, *a1, *a2, *a3, *P;       // plain FP64 form
  float *uf, *vf, *wf, *a1f, *a2f, *a3f, *Pf;  // precision form
  long long *pid;
  int *cell;
  unsigned char *status;
};

// Division by a fixed divisor d >= 1 for numerators n < 2^31 (cell and node
// indices): floor(n/d) = (n * m) >> (31 + s) with s = ceil(log2 d) and
// m = ceil(2^(31+s) / d) < 2^32.  Exact: m*n/2^(31+s) exceeds n/d by less than
// 2^-s <= 1/d, which cannot carry past the next integer (equality only for
// d = 2^s, where m is exact).
struct FastDiv {
  unsigned int d, m;
  int sh;
  __host__ void init(unsigned int div) {
    d = div;
    int s = 0;
    while ((1ull << s) < (unsigned long long)div) ++s;
    sh = 31 + s;
    unsigned long long num = 1ull << sh;
    m = (unsigned int)((num + div - 1) / div);
  }
  __device__ __forceinline__ unsigned int div(unsigned int n) const {
    return (unsigned int)(((unsigned long long)n * m) >> sh);
  }
};

struct GridDims {
  int IM, JM, KM;
  long long Nc, Nn;
  FastDiv fIM, fJM, fMX, fMY;   // by IM, JM (cells) and IM+1, JM+1 (nodes)
};

// cell id -> (i, j, k)
__device__ __forceinline__ void cell_ijk(const GridDims &g, unsigned int c, int &i, int &j, int &k) {
  unsigned int t = g.fIM.div(c);
  i = (int)(c - t * (unsigned)g.IM);
  unsigned int kk = g.fJM.div(t);
  j = (int)(t - kk * (unsigned)g.JM);
  k = (int)kk;
}
// node id -> (i, j, k)
__device__ __forceinline__ void node_ijk(const GridDims &g, unsigned int q, int &i, int &j, int &k) {
  unsigned int t = g.fMX.div(q);
  i = (int)(q - t * (unsigned)(g.IM + 1));
  unsigned int kk = g.fMY.div(t);
  j = (int)(t - kk * (unsigned)(g.JM + 1));
  k = (int)kk;
}

// Threads per block of the advect + locate kernels.  A block keeps its SM slot until its
// slowest walk ends, so smaller blocks waste fewer warp slots on the walk-length tail (FP32 walk
// per 64M-particle step at 1152 resident threads: 3.15 ms in 64-thread blocks, 3.17 in 128, 3.18
// in 96, 3.42 in 256).
#ifndef FDF_LOC_THREADS
#define FDF_LOC_THREADS 64
#endif
// Resident blocks per SM the FP32 locate kernels are compiled for.  The walk is bound by load
// latency, so resident threads beat spills up to a point: with 176-B plane-table rows 1024
// threads (64 registers) beat 768 (80): 3.9 against 4.8 ms per 64M-particle step, and 1280 (48
// registers) spilled too much; with the 128-B rows 1152 threads (56 registers, a few more spills)
// take 3.17 against 3.22 ms for the FP32 walk.
#ifndef FDF_LOC_MIN_BLOCKS
#define FDF_LOC_MIN_BLOCKS (1152 / FDF_LOC_THREADS)
#endif
// Resident blocks per SM of the plain walk (its steps decided from the FP32 table; per
// 64M-particle step 1024 resident threads take 7.6 ms against 8.6 ms at 768 and 8.4 ms at 1280
// or 1536, where spills grow) and of the per-cell PID ordering (latency-bound: 2048 resident threads at 32 registers,
// 1.59 -> 1.24 ms for the 64M-particle sort stage).
#ifndef FDF_PLAIN_MIN_BLOCKS
#define FDF_PLAIN_MIN_BLOCKS 8
#endif
// Threads per block of the plain walk (with FDF_PLAIN_MIN_BLOCKS: 1024 resident threads).
#ifndef FDF_PLAIN_THREADS
#define FDF_PLAIN_THREADS 128
#endif
#ifndef FDF_ORDER_MIN_BLOCKS
#define FDF_ORDER_MIN_BLOCKS 8
#endif
// Resident 256-thread blocks per SM the learned form's walk from P1 is compiled for (4: 64
// registers, 0.701 ms per 64M-particle step against 0.712 ms at 3 with 80 registers).
#ifndef FDF_GUESS_MIN_BLOCKS
#define FDF_GUESS_MIN_BLOCKS 4
#endif
// Threads per block of the learned form's walk from P1.
#ifndef FDF_GUESS_THREADS
#define FDF_GUESS_THREADS 256
#endif

// ---------------------------------------------------------------- kernels (launchers)
// Compaction of the held swarm to slots [a, b) and [c, n) of src, in that order (fdf_ExtractParticles).
void launch_move_kept(const SwarmBuf &src, const SwarmBuf &dst, int a, int b, int c, int n, cudaStream_t s);
// The plain form's k-faces of layer k summed again from seeds (fdf_DepositKFaceLayer).
void launch_deposit_k_layer(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, int k, double volume,
                            const double *seed, const double *seed_mom, double *fk, double *mk, cudaStream_t s);
// Adds the pending block flushes to the counters and clears them (end of a pipeline run).
void launch_fold_counts(DevCounters *cnt, cudaStream_t s);
void launch_build_planes(const double *coor_aos, GridDims g, double *planes, unsigned int *err, cudaStream_t s);
// cell_start == nullptr: every node; else only nodes adjacent to an occupied cell.
void launch_center_to_corner(const double *ucat, GridDims g, double *corner, const unsigned int *cell_start,
                             unsigned long long *nodes_done, cudaStream_t s);
// Advect + walk.  Writes the new cell (or -1) and status in place, keys[s] = cell
// or sentinel (LOST / removed), and histograms the kept keys into count[] (bucket
// Nc = LOST particles, counted only when keep_lost), with rank[s] = the particle's rank
// among its key's particles (rank may be null).
// table: the FP32 plane table, which decides the walk's steps exactly.
void launch_locate(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes, double dt,
                   int advect, const double *bbox, int drop_removed, DevCounters *cnt, unsigned int *keys,
                   unsigned int *rank, unsigned int *count, unsigned int sentinel, cudaStream_t s);
// Modes of the gather kernels: sorted slot s takes the particle perm[s] (perm == nullptr: s
// itself, src == dst allowed) for s < n = cell_start[Nc+1] (read on the device), and
//   GATHER_INTERP  interpolates its velocity and sets its status from its cell (the step),
//   GATHER_COPY    copies velocity and status (a re-sort or a removal),
//   INTERP_KEEP    interpolates its velocity and keeps its status (InterpolateAllFieldsToSwarm).
enum { GATHER_COPY = 0, GATHER_INTERP = 1, INTERP_KEEP = 2 };
void launch_gather_interp(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g,
                          const double *corner, const unsigned int *perm, const unsigned int *cell_start,
                          DevCounters *cnt, cudaStream_t s, int mode = GATHER_INTERP);
// mi, mj, mk (SoA [3][faces], or nullptr): the momentum deposit, V * velocity split like the volume.
void launch_deposit(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, double volume, double *count,
                    double *avg, double *fi, double *fj, double *fk, double *mi, double *mj, double *mk,
                    cudaStream_t s);

// Counting sort helpers (fdf_sort.cu).
size_t scan_scratch_words(long long count);
long long scan_max_count();
void exclusive_scan_u32(unsigned int *data, long long count, unsigned int *sums, cudaStream_t s);
// perm[cell_start[key] + rank[s]] = s for every kept particle (keys and ranks from the locate
// kernels' histogram).
void launch_scatter_slots(const unsigned int *keys, const unsigned int *rank, int n_cap, const DevCounters *cnt,
                          unsigned int sentinel, int keep_lost, const unsigned int *cell_start, unsigned int *perm,
                          cudaStream_t s);
void launch_order_segments(const unsigned int *cell_start, int nseg, const long long *pid, unsigned int *perm,
                           cudaStream_t s);
void cell_sort_on_scratch(const int *cell, long long n, long long ncells, unsigned int *perm,
                          unsigned int *cell_start, unsigned int *cursor, unsigned int *sums, cudaStream_t s);

// AoS <-> SoA marshalling of the DMSwarm fields.
void launch_swarm_from_aos(const double *pos, const double *vel, const double *wgt, const double *P,
                           const long long *cell3, const long long *pid, const long long *status, int n,
                           GridDims g, const SwarmBuf &b, cudaStream_t s);
void launch_swarm_to_aos(const SwarmBuf &b, int n, GridDims g, double *pos, double *vel, double *wgt,
                         double *P, long long *cell3, long long *pid, long long *status, cudaStream_t s);

// The reference's stages one at a time (ParticleMotion.c): status reset, position update
// (plain and precision forms), and the sort keys of a re-sort that may drop the LOST and/or the
// out-of-bounds particles (either form; ranks and histogram as the locate kernels make them).
void launch_reset_status(const SwarmBuf &b, int n_cap, const DevCounters *cnt, cudaStream_t s);
void launch_advect(const SwarmBuf &b, int n_cap, double dt, DevCounters *cnt, cudaStream_t s);
void launch_advect32(const SwarmBuf &b, int n_cap, double dt, DevCounters *cnt, cudaStream_t s);
void launch_resort_keys(const SwarmBuf &b, int n_cap, GridDims g, int f32, int remove_lost, int remove_oob,
                        const double *bbox, const float *fbox, DevCounters *cnt, unsigned int *keys,
                        unsigned int *rank, unsigned int *count, unsigned int sentinel, cudaStream_t s);

// Precision form (fdf_fp32.cu).
void launch_build_table32(const double *planes, const double *coor, GridDims g, float *table, cudaStream_t s);
// fbox: 12 floats, (x, y, z, -) lower and (x, y, z, -) upper bounds strictly inside the
// bounding box by more than any lo part of a position inside it, then 4 unused.
// pending != nullptr: the learned form's first pass (one evaluation in the previous cell;
// pending[s] = 1 for the particles that leave it by at least far_cells cells, 0 otherwise,
// for s <= n_cap; the others are located here).
void launch_locate32(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes, double dt,
                     int advect, const double *bbox, const float *fbox, int drop_removed, DevCounters *cnt,
                     unsigned int *keys, unsigned int *rank, unsigned int *count, unsigned int sentinel,
                     unsigned int *pending, float far_cells, cudaStream_t s);
// The learned form's pending list from the warps' masks and scanned counts (sets cnt->pending).
void launch_compact_pending(const unsigned int *scan, int n_cap, unsigned int *list, DevCounters *cnt,
                            cudaStream_t s);
// The learned form's second pass over pending[0 .. cnt->pending): the reference walk from P1 (the
// particle's cell field), with the table rows of the path toward guess[t] prefetched.
void launch_locate32_path(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes,
                          const double *bbox, const float *fbox, int drop_removed, DevCounters *cnt,
                          unsigned int *keys, unsigned int *rank, unsigned int *count, unsigned int sentinel,
                          const unsigned int *pending, const int *guess, int num_sms, cudaStream_t s);
void launch_center_to_corner32(const float *ucat, GridDims g, float *corner, const unsigned int *cell_start,
                               unsigned long long *nodes_done, cudaStream_t s);
void launch_gather_interp32(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g, const float *corner,
                            const unsigned int *perm, const unsigned int *cell_start, DevCounters *cnt,
                            cudaStream_t s, int mode = GATHER_INTERP);
void launch_deposit32(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, double volume, float *count,
                      float *avg, float *fi, float *fj, float *fk, float *mi, float *mj, float *mk, cudaStream_t s);
void launch_swarm_from_aos32(const double *pos, const double *vel, const double *wgt, const double *P,
                             const long long *cell3, const long long *pid, const long long *status, int n, GridDims g,
                             const SwarmBuf &b, cudaStream_t s);
void launch_swarm_to_aos32(const SwarmBuf &b, int n, GridDims g, double *pos, double *vel, double *wgt, double *P,
                           long long *cell3, long long *pid, long long *status, cudaStream_t s);
// The layout conversion straight from / to page-locked host DMSwarm arrays (device addresses,
// 16-byte aligned; f = position, velocity, weight, P, cell, pid, status), either form.
void launch_swarm_from_host(const void *const f[7], int n, GridDims g, const SwarmBuf &b, bool f32, cudaStream_t s);
void launch_swarm_to_host(const SwarmBuf &b, int n, GridDims g, void *const f[7], bool f32, cudaStream_t s);
void launch_f64_to_f32(const double *in, float *out, long long n, cudaStream_t s);
void launch_f32_to_f64(const float *in, double *out, long long n, cudaStream_t s);

// On-device volumetric seeding (fdf_seed.cu), bit-identical to the host generator.
void launch_seed(const double *coor, GridDims g, long long n, unsigned long long seed, long long pid_base, int hint,
                 int form32, double P0, const SwarmBuf &b, cudaStream_t s);
