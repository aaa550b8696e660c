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
#define FDF_MAX_TRAVERSAL 1000
#define FDF_DISTANCE_THRESHOLD 1e-11
#define FDF_INTERP_DIST_TOL 1e-14
#define FDF_BBOX_TOL 1e-6

// Face order of the reference (common.h Face enum).
enum { F_LEFT = 0, F_RIGHT = 1, F_BOTTOM = 2, F_TOP = 3, F_FRONT = 4, F_BACK = 5 };
// Particle status values of the reference (common.h ParticleLocationStatus).
enum { ST_NEEDS_LOCATION = 0, ST_ACTIVE_AND_LOCATED = 1, ST_MIGRATING_OUT = 2, ST_LOST = 3,
       ST_UNINITIALIZED = 4 };

// Device error word bits.
enum { ERRBIT_DEGENERATE = 1u, ERRBIT_BAD_CELL = 2u };

// Counters kept on the device so that a step needs no host round trip.
struct DevCounters {
  unsigned long long removed_lost;
  unsigned long long removed_oob;
  unsigned long long evals;        // walk evaluations the reference makes for this run (cycles count MAX_TRAVERSAL)
  unsigned long long lost_total;
  unsigned int err;
  unsigned int pad;
  int n;            // live particle count after the last removal
  int n_sorted;     // particles held in the arrays (live + LOST kept by the initial setup)
  unsigned long long psteps_total;  // sum over steps of the particles at step start (never reset per step)
  unsigned long long evals_total;   // walk evaluations actually made, all pipeline runs (never reset per step)
};

struct SwarmBuf {
  double *x, *y, *z, *u, *v, *w, *a1, *a2, *a3, *P;
  long long *pid;
  int *cell;
  unsigned char *status;
};

struct GridDims {
  int IM, JM, KM;
  long long Nc, Nn;
};

// ---------------------------------------------------------------- kernels (launchers)
void launch_build_planes(const double *coor_aos, GridDims g, double *planes, unsigned int *err, cudaStream_t s);
void launch_center_to_corner(const double *ucat, GridDims g, double *corner, cudaStream_t s);
void launch_locate(const SwarmBuf &b, int n_cap, GridDims g, const double *planes, double dt, int advect,
                   const double *bbox, int drop_removed, DevCounters *cnt, unsigned int *keys,
                   unsigned int *vals, unsigned int sentinel, cudaStream_t s);
void launch_gather_interp(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g,
                          const double *corner, const unsigned int *keys, const unsigned int *vals,
                          unsigned int sentinel, const DevCounters *cnt, cudaStream_t s);
void launch_update_counts(DevCounters *cnt, const int *cell_start, unsigned int sentinel, int drop_removed,
                          cudaStream_t s);
void launch_cell_bounds(const unsigned int *keys, int n_cap, const DevCounters *cnt, unsigned int sentinel,
                        int *cell_start, cudaStream_t s);
void launch_deposit(const SwarmBuf &b, GridDims g, const int *cell_start, double volume, double *count,
                    double *avg, double *fi, double *fj, double *fk, cudaStream_t s);
void launch_bbox(const double *coor_aos, long long nn, double *bbox6, cudaStream_t s);

// Radix sort of (key, value) pairs, stable, ascending, on the low `bits` bits of the key.
struct RadixScratch {
  unsigned int *keys_alt, *vals_alt, *hist, *hist_scan_tmp;
  int cap_items, cap_tiles;
};
size_t radix_scratch_bytes(int n_cap);
void radix_scratch_carve(void *base, int n_cap, RadixScratch *rs);
// Sorts (*keys, *vals); n is read from *n_dev on the device.  The passes ping-pong
// with rs.keys_alt/vals_alt: on return *keys/*vals point at the sorted pairs and
// rs.keys_alt/vals_alt at the other buffers.
void radix_sort_pairs(unsigned int **keys, unsigned int **vals, const int *n_dev, int bits, RadixScratch &rs,
                      cudaStream_t s);

// AoS <-> SoA marshalling of the DMSwarm fields.
void launch_swarm_from_aos(const double *pos, const double *vel, const double *wgt, const double *P,
                           const long long *cell3, const long long *pid, const long long *status, int n,
                           GridDims g, const SwarmBuf &b, cudaStream_t s);
void launch_swarm_to_aos(const SwarmBuf &b, int n, GridDims g, double *pos, double *vel, double *wgt,
                         double *P, long long *cell3, long long *pid, long long *status, cudaStream_t s);
