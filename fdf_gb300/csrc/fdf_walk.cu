// fdf_walk.cu -- fused advect + walking-search locate, one thread per particle.
//
// Restates, per particle, UpdateParticlePosition (ParticleMotion.c:19-29) and
// LocateParticleOrFindMigrationTarget_TEST (walkingsearch.c:1094-1242) with
// EvaluateParticlePosition (:811-859), DeterminePointPosition (:407-462),
// UpdateCellIndicesBasedOnDistancesTEST (:882-959) and UpdateParticleWeights
// (ParticleSwarm.c:1010-1047).  The per-cell plane table holds every
// particle-independent value of ComputeSignedDistanceToPlane, computed with the
// reference's own operation order, so each signed distance here is the
// reference's bit for bit: d = (fc - p) . n, then |d| < thr -> 0.
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

namespace {

using fdfx::add;
using fdfx::sub;
using fdfx::mul;

__global__ void __launch_bounds__(FDF_LOC_THREADS, FDF_PLAIN_MIN_BLOCKS) k_locate(SwarmBuf b, GridDims g, const double *__restrict__ planes,
                                                double dt, int advect, int reset_first, const double *__restrict__ bbox,
                                                int drop_removed, DevCounters *cnt, unsigned int *__restrict__ keys,
                                                unsigned int *__restrict__ rank, unsigned int *__restrict__ count,
                                                unsigned int sentinel) {
  const int n = cnt->n_sorted;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0 && advect) atomicAdd(&cnt->psteps_total, (unsigned long long)n);
  unsigned int my_lost = 0, my_oob = 0, my_evals = 0, my_done = 0, my_lost_total = 0;
  unsigned int my_err = 0;
  unsigned int hkey = 0xffffffffu;   // histogram bucket of this particle (none = all ones)
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
      // InitializeTraversalParameters: previous cell if it is inside the grid, else (0,0,0)
      int i = 0, j = 0, k = 0;
      if (cell >= 0 && (long long)cell < g.Nc) cell_ijk(g, (unsigned int)cell, i, j, k);
      int steps = 0, evaluated = 0;
      bool concluded = false, cycle = false;
      long long saved = -1;
      int power = 1, lam = 0;
      double d[6];
      while (!concluded && steps < FDF_MAX_TRAVERSAL) {
        ++steps;
        if (i < 0 || i >= g.IM || j < 0 || j >= g.JM || k < 0 || k >= g.KM) { lost = true; break; }
        const long long cur = ((long long)k * g.JM + j) * g.IM + i;
        if (cur == saved) { cycle = true; lost = true; break; }
        if (++lam == power) { saved = cur; power <<= 1; lam = 0; }
        const double2 *row = reinterpret_cast<const double2 *>(planes + cur * FDF_ROW);
        double2 tf = __ldg(row + 18);   // thr, degenerate flag
        if (fdfx::ubits(tf.y) != 0ULL) { my_err |= ERRBIT_DEGENERATE; lost = true; break; }
        const unsigned long long thr_bits = fdfx::ubits(tf.x);
        const bool thr_nan = fdfx::is_nan(tf.x);
        ++evaluated;
        bool neg = false, zero = false;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
          double2 p0 = __ldg(row + 3 * f), p1 = __ldg(row + 3 * f + 1), p2 = __ldg(row + 3 * f + 2);
          // p0 = (fc.x, fc.y), p1 = (fc.z, n.x), p2 = (n.y, n.z); d = (fc - p) . n
          double dd = add(add(mul(sub(p0.x, x), p1.y), mul(sub(p0.y, y), p2.x)), mul(sub(p1.x, z), p2.y));
          if (fdfx::abs_lt_bits(dd, thr_bits, thr_nan)) dd = 0.0;
          d[f] = dd;
          neg |= fdfx::lt0(dd);
          zero |= fdfx::eq0(dd);
        }
        if (!neg || zero) {
          concluded = true;   // position >= 0: inside, or on a face (accepted even if outside another)
        } else {
          if (fdfx::lt0(d[F_FRONT])) k += 1; else if (fdfx::lt0(d[F_BACK])) k -= 1;
          if (fdfx::lt0(d[F_LEFT])) i -= 1; else if (fdfx::lt0(d[F_RIGHT])) i += 1;
          if (fdfx::lt0(d[F_BOTTOM])) j -= 1; else if (fdfx::lt0(d[F_TOP])) j += 1;
        }
      }
      my_evals = (unsigned long long)(cycle ? FDF_MAX_TRAVERSAL : steps);
      my_done = (unsigned long long)evaluated;
      if (lost || !concluded) {
        lost = true;
        cell = -1;
        st = ST_LOST;
      } else {
        const unsigned long long tol_bits = fdfx::ubits(FDF_INTERP_DIST_TOL);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fdfx::le_pos(d[f], tol_bits)) d[f] = FDF_INTERP_DIST_TOL;
        b.a1[s] = __ddiv_rn(d[F_LEFT], add(d[F_LEFT], d[F_RIGHT]));
        b.a2[s] = __ddiv_rn(d[F_BOTTOM], add(d[F_BOTTOM], d[F_TOP]));
        b.a3[s] = __ddiv_rn(d[F_BACK], add(d[F_FRONT], d[F_BACK]));
        cell = (int)(((long long)k * g.JM + j) * g.IM + i);
        st = ST_ACTIVE_AND_LOCATED;
      }
      b.cell[s] = cell;
      b.status[s] = st;
    } else {
      lost = (cell < 0);
    }
    unsigned int key = lost ? sentinel : (unsigned int)cell;
    if (lost) my_lost_total = 1;
    if (drop_removed) {
      // CheckAndRemoveLostParticles, then CheckAndRemoveOutOfBoundsParticles on the rest.
      if (lost) {
        my_lost = 1;
      } else {
        bool inside = x >= bbox[0] && x <= bbox[3] && y >= bbox[1] && y <= bbox[4] && z >= bbox[2] && z <= bbox[5];
        if (!inside) { my_oob = 1; key = sentinel; }
      }
    }
    keys[s] = key;
    if (key < sentinel) hkey = key;
    else if (!drop_removed) hkey = sentinel;   // the initial setup keeps LOST particles, at the end
  }
  const unsigned int r = warp_histogram_rank(hkey, count);
  if (rank && hkey != 0xffffffffu) rank[s] = r;
  LocCounts m;
  m.lost = my_lost; m.oob = my_oob; m.evals = my_evals; m.done = my_done; m.lost_total = my_lost_total;
  m.err = my_err;
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

void launch_locate(const SwarmBuf &b, int n_cap, GridDims g, const double *planes, double dt, int advect,
                   const double *bbox, int drop_removed, DevCounters *cnt, unsigned int *keys, unsigned int *rank,
                   unsigned int *count, unsigned int sentinel, cudaStream_t s) {
  // advect and drop_removed are both set by the fused step, which also resets statuses first.
  int reset_first = drop_removed;
  constexpr int th = FDF_LOC_THREADS;
  int blocks = (n_cap + th - 1) / th;
  if (blocks == 0) blocks = 1;
  k_locate<<<blocks, th, 0, s>>>(b, g, planes, dt, advect, reset_first, bbox, drop_removed, cnt, keys, rank, count,
                                 sentinel);
}
