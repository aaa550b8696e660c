// fdf_walk.cu -- fused advect + walking-search locate, one thread per particle.
//
// Restates, per particle, UpdateParticlePosition (ParticleMotion.c:19-29) and
// LocateParticleOrFindMigrationTarget_TEST (walkingsearch.c:1094-1242) with
// EvaluateParticlePosition (:811-859), DeterminePointPosition (:407-462),
// UpdateCellIndicesBasedOnDistancesTEST (:882-959) and UpdateParticleWeights
// (ParticleSwarm.c:1010-1047).  The per-cell plane table holds every
// particle-independent value of ComputeSignedDistanceToPlane, computed with the
// reference's own operation order, so each FP64 signed distance here is the
// reference's bit for bit: d = (fc - p) . n, then |d| < thr -> 0.
//
// The walk's steps take their face classes from the FP32 plane table with a rigorous
// error bound and fall back to the FP64 distance of a face only where the bound cannot
// decide (fdf_walk.cuh), so the path of cells is the FP64 walk's; the concluding cell's
// six distances are computed in FP64 as the reference computes them, for the weights.
// Positions, velocities and weights are the reference's bit for bit; what goes is the
// FP64 work of every evaluation before the last.
//
// The stuck-cell tie-breaker (walkingsearch.c:1149-1185) cannot fire on one
// rank: an evaluation either concludes (position >= 0) or reports some d < 0,
// and UpdateCellIndices then changes at least one index, so the same cell is
// never visited twice in a row.  It is therefore not restated here.
//
// Cycle cut-off.  The next cell of the walk is a function of (cell, position)
// only, so once the walk returns to a cell it has already evaluated without
// concluding, it repeats that cycle until MAX_TRAVERSAL and the particle is
// LOST.  This happens for points in the thin gap between a cell's FRONT plane
// and the next cell's BACK plane on curved grids (the two planes are built from
// different corner vertices, walkingsearch.c:303-325).  The walk here detects
// the revisit (Brent's method: compare with the cell saved at step 2^m) and
// concludes LOST at once; the outcome, cell (-1,-1,-1), and the unchanged
// weights are the reference's, and the evaluation count reported for parity is
// the reference's (MAX_TRAVERSAL).
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"
#include "fdf_counters.cuh"
#include "fdf_walk.cuh"

namespace {

using fdfx::add;
using fdfx::sub;
using fdfx::mul;

__global__ void __launch_bounds__(FDF_PLAIN_THREADS, FDF_PLAIN_MIN_BLOCKS)
    k_locate(SwarmBuf b, GridDims g, const float *__restrict__ table, const double *__restrict__ planes, double dt,
               int advect, int reset_first, const double *__restrict__ bbox, int drop_removed, DevCounters *cnt,
               unsigned int *__restrict__ keys, unsigned int *__restrict__ rank, unsigned int *__restrict__ count,
               unsigned int sentinel) {
  const int n = cnt->n_sorted;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0 && advect) atomicAdd(&cnt->psteps_total, (unsigned long long)n);
  LocCounts m;
  unsigned int hkey = 0xffffffffu;
  if (s < n) {
    double x = b.x[s], y = b.y[s], z = b.z[s];
    if (advect) {
      x = add(x, mul(b.u[s], dt));
      y = add(y, mul(b.v[s], dt));
      z = add(z, mul(b.w[s], dt));
      b.x[s] = x; b.y[s] = y; b.z[s] = z;
    }
    unsigned char st = b.status[s];
    if (reset_first && st == ST_ACTIVE_AND_LOCATED) st = ST_NEEDS_LOCATION;
    int cell = b.cell[s];
    bool lost = false;
    if (st != ST_ACTIVE_AND_LOCATED) {
      // (hi, lo) within 2^-48 |v| of v; a nonzero |v| below 2^-120 (where the split's error is
      // absolute) gives a NaN pair, whose faces all take the FP64 route
      auto split = [](double v) {
        const unsigned long long mag = fdfx::ubits(v) & fdfx::ABS_MASK;
        if (mag < (903ull << 52) && mag != 0ull) return make_float2(__int_as_float(0x7fc00000), 0.f);
        return fdfx::split_rn(v);
      };
      Walk32 w;
      w.i = 0; w.j = 0; w.k = 0; w.err = 0u;   // InitializeTraversalParameters: previous cell, else (0,0,0)
      if (cell >= 0 && (long long)cell < g.Nc) cell_ijk(g, (unsigned int)cell, w.i, w.j, w.k);
      walk_ref32<true>(table, planes, g, split(x), split(y), split(z), FDF_MAX_TRAVERSAL, w, m.fb, x, y, z);
      m.err |= w.err;
      m.evals += (unsigned int)(w.cycle ? FDF_MAX_TRAVERSAL : w.steps);
      m.done += (unsigned int)w.evaluated;
      if (w.lost || !w.concluded) {
        lost = true;
        cell = -1;
        st = ST_LOST;
      } else {
        cell = (int)(((long long)w.k * g.JM + w.j) * g.IM + w.i);
        const double *row = planes + (long long)cell * FDF_ROW;
        double d[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) d[f] = exact_face(row, f, x, y, z);
        const unsigned long long tol_bits = fdfx::ubits(FDF_INTERP_DIST_TOL);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fdfx::le_pos(d[f], tol_bits)) d[f] = FDF_INTERP_DIST_TOL;
        b.a1[s] = fdfx::div_rn(d[F_LEFT], add(d[F_LEFT], d[F_RIGHT]));
        b.a2[s] = fdfx::div_rn(d[F_BOTTOM], add(d[F_BOTTOM], d[F_TOP]));
        b.a3[s] = fdfx::div_rn(d[F_BACK], add(d[F_FRONT], d[F_BACK]));
        st = ST_ACTIVE_AND_LOCATED;
      }
      b.cell[s] = cell;
      b.status[s] = st;
    } else {
      lost = (cell < 0);
    }
    unsigned int key = lost ? sentinel : (unsigned int)cell;
    if (lost) m.lost_total += 1;
    if (drop_removed) {   // CheckAndRemoveLostParticles, then CheckAndRemoveOutOfBoundsParticles
      if (lost) {
        m.lost += 1;
      } else {
        // IsParticleInBox, the six comparisons on the integer pipe
        const bool inside = fdfx::in_range(x, bbox[0], bbox[3]) && fdfx::in_range(y, bbox[1], bbox[4]) &&
                            fdfx::in_range(z, bbox[2], bbox[5]);
        if (!inside) { m.oob += 1; key = sentinel; }
      }
    }
    keys[s] = key;
    if (key < sentinel) hkey = key;
    else if (!drop_removed) hkey = sentinel;   // the initial setup keeps LOST particles, at the end
  }
  const unsigned int r = warp_histogram_rank(hkey, count);
  if (rank && hkey != 0xffffffffu) rank[s] = r;
  block_flush_counts(m, cnt);
}

// One warp per flush slot: sums the slot over the rows, clears them, and adds the sum to its
// counter(s).  Integer sums, so the totals do not depend on the flush order.
__global__ void k_fold_counts(DevCounters *cnt) {
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
  if (q > CNT_FB) return;
  unsigned long long t = 0;
  for (int r = lane; r < FDF_CNT_STRIPES; r += 32) {
    t += cnt->stripes[r][q];
    cnt->stripes[r][q] = 0ull;
  }
  t = warp_sum_u64(t);
  if (lane == 0 && t) {
    switch (q) {
      case CNT_LOST: cnt->removed_lost += t; break;
      case CNT_OOB: cnt->removed_oob += t; break;
      case CNT_EVALS: cnt->evals += t; break;
      case CNT_EVALS_TOTAL: cnt->evals_total += t; break;
      case CNT_LOST_TOTAL: cnt->lost_total += t; break;
      default: cnt->fallbacks += t; cnt->fallbacks_total += t; break;
    }
  }
}

}  // namespace

void launch_fold_counts(DevCounters *cnt, cudaStream_t s) { k_fold_counts<<<1, 32 * (CNT_FB + 1), 0, s>>>(cnt); }

void launch_locate(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes, double dt,
                   int advect, const double *bbox, int drop_removed, DevCounters *cnt, unsigned int *keys,
                   unsigned int *rank, unsigned int *count, unsigned int sentinel, cudaStream_t s) {
  // advect and drop_removed are both set by the fused step, which also resets statuses first
  constexpr int th = FDF_PLAIN_THREADS;
  const unsigned int blocks = n_cap > 0 ? (unsigned int)((n_cap + th - 1) / th) : 1u;
  k_locate<<<blocks, th, 0, s>>>(b, g, table, planes, dt, advect, drop_removed, bbox, drop_removed, cnt,
                                                keys, rank, count, sentinel);
}
