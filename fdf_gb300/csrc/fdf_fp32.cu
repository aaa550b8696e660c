// fdf_fp32.cu -- the precision form: interpolation, advection and deposition in FP32,
// cell location decided exactly as the FP64 reference walk decides it.
//
// Positions.  The form holds each coordinate as a float pair (hi, lo) with |lo| <=
// ulp(hi)/2; the form's position is the exact sum hi + lo (a double).  Advection adds
// the FP32 displacement fl32(u * dt) by double-float addition (FP32 operations only).
// Uploads split the caller's FP64 position (an error of at most 2^-48 |p|); downloads
// return hi + lo exactly.
//
// Walk.  Every face class the walk needs is decided exactly as the FP64 reference decides it
// (fdf_walk.cuh: the FP32 plane table with a rigorous error bound, FP64 where it cannot
// decide), so the cells, statuses and walk paths are the reference's for the form's own
// positions.
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"
#include "fdf_counters.cuh"
#include "fdf_walk.cuh"

namespace {

using fdfx::add;
using fdfx::mul;
using fdfx::sub;

// One 128-B FP32 row per cell (the layout and the error bound are in fdf_walk.cuh): the first
// vertex c0 as a float pair, thr32, the absolute slack for the FP64 arithmetic of the table, then
// per face n32 = fl32(n) and e32 = fl32(n . (fc - c0)).
__global__ void k_build_table32(const double *__restrict__ planes, const double *__restrict__ coor, GridDims g,
                                float *__restrict__ table) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= g.Nc) return;
  int i, j, k;
  cell_ijk(g, (unsigned int)c, i, j, k);
  const double *v0 = coor + 3 * (((long long)k * (g.JM + 1) + j) * (long long)(g.IM + 1) + i);
  const double *row = planes + c * FDF_ROW;
  float *t = table + c * FDF_ROW32;
  double c0[3];
  for (int q = 0; q < 3; ++q) {
    const float h = __double2float_rn(v0[q]);
    const float l = __double2float_rn(sub(v0[q], (double)h));
    t[q] = h;
    t[4 + q] = l;
    c0[q] = add((double)h, (double)l);   // exact: the pair's value
  }
  const double thr = row[36];
  // rounded up with a little headroom: thr32 * (1 - 2^-24)^2 >= thr, which the error bound uses;
  // a degenerate cell carries the sign bit
  float thr32 = __double2float_ru(mul(thr, 1.0 + 0x1p-22));
  if (fdfx::ubits(row[37]) != 0ULL) thr32 = -fabsf(thr32) - 1.0f;
  t[3] = thr32;
  double sigma = 0.0;   // max over faces of sum_i |fc_i - c0_i| |n_i|
  for (int f = 0; f < 6; ++f) {
    const double *p = row + 6 * f;
    const double dx = sub(p[0], c0[0]), dy = sub(p[1], c0[1]), dz = sub(p[2], c0[2]);
    const double e = add(add(mul(dx, p[3]), mul(dy, p[4])), mul(dz, p[5]));
    const double sg = add(add(mul(fabs(dx), fabs(p[3])), mul(fabs(dy), fabs(p[4]))), mul(fabs(dz), fabs(p[5])));
    sigma = sg > sigma ? sg : sigma;
    float *o = t + 8 + 4 * f;
    o[0] = __double2float_rn(p[3]);
    o[1] = __double2float_rn(p[4]);
    o[2] = __double2float_rn(p[5]);
    o[3] = __double2float_rn(e);
  }
  // the FP64 roundings of e and of the reference's own distance, 32 eps sigma (rounded up)
  t[7] = __double2float_ru(mul(sigma, 0x1p-48));
}

// (hi, lo) float pair held in a double slot of the swarm arrays
__device__ __forceinline__ float2 ld_pair(const double *a, int s) {
  return *reinterpret_cast<const float2 *>(a + s);
}
__device__ __forceinline__ void st_pair(double *a, int s, float2 v) { *reinterpret_cast<float2 *>(a + s) = v; }

// (hi, lo) + v for a float v (double-float addition, FP32 operations only).
__device__ __forceinline__ float2 pair_add(float2 p, float v) {
  const float sh = __fadd_rn(p.x, v);
  const float bv = __fsub_rn(sh, p.x);
  const float e = __fadd_rn(__fsub_rn(p.x, __fsub_rn(sh, bv)), __fsub_rn(v, bv));   // exact error of p.x + v
  const float t = __fadd_rn(p.y, e);
  const float h = __fadd_rn(sh, t);
  return make_float2(h, __fsub_rn(t, __fsub_rn(h, sh)));
}


// Writes the located (or LOST) particle: weights (UpdateParticleWeights in FP32: clamp
// d <= 1e-14, then the three ratios), cell and status.
__device__ __forceinline__ void store_located32(const SwarmBuf &b, int s, const GridDims &g, bool lost, int i, int j,
                                                int k, float (&dv)[6]) {
  if (lost) {
    b.cell[s] = -1;
    b.status[s] = ST_LOST;
    return;
  }
#pragma unroll
  for (int f = 0; f < 6; ++f)
    if (!(dv[f] > 1e-14f)) dv[f] = (dv[f] != dv[f]) ? dv[f] : 1e-14f;
  b.a1f[s] = __fdiv_rn(dv[F_LEFT], __fadd_rn(dv[F_LEFT], dv[F_RIGHT]));
  b.a2f[s] = __fdiv_rn(dv[F_BOTTOM], __fadd_rn(dv[F_BOTTOM], dv[F_TOP]));
  b.a3f[s] = __fdiv_rn(dv[F_BACK], __fadd_rn(dv[F_FRONT], dv[F_BACK]));
  b.cell[s] = (int)(((long long)k * g.JM + j) * g.IM + i);
  b.status[s] = ST_ACTIVE_AND_LOCATED;
}

// Sort key of a particle whose location is final, with IsParticleInBox on the form's
// position: decided in FP32 when the hi parts are clear of the box faces by more than the
// lo parts and rounding can move them (fbox = the box shrunk accordingly), exactly in
// FP64 otherwise.
__device__ __forceinline__ unsigned int settle_key32(bool lost, int cell, float2 px, float2 py, float2 pz,
                                                     int drop_removed, const double *__restrict__ bbox,
                                                     const float *__restrict__ fbox, unsigned int sentinel,
                                                     unsigned int &my_lost, unsigned int &my_oob,
                                                     unsigned int &my_lost_total) {
  unsigned int key = lost ? sentinel : (unsigned int)cell;
  if (lost) my_lost_total += 1;
  if (drop_removed) {
    if (lost) {
      my_lost += 1;
    } else {
      const float4 fb0 = *reinterpret_cast<const float4 *>(fbox), fb1 = *reinterpret_cast<const float4 *>(fbox + 4);
      const bool surely_in = px.x > fb0.x && px.x < fb1.x && py.x > fb0.y && py.x < fb1.y && pz.x > fb0.z &&
                             pz.x < fb1.z;
      bool inside = surely_in;
      if (!surely_in) {
        const double x = pair_value(px), y = pair_value(py), z = pair_value(pz);
        inside = x >= bbox[0] && x <= bbox[3] && y >= bbox[1] && y <= bbox[4] && z >= bbox[2] && z <= bbox[5];
      }
      if (!inside) { my_oob += 1; key = sentinel; }
    }
  }
  return key;
}

// How far past the previous cell a particle is, in cells, from the first evaluation's
// distances: for each index direction with a negative face, -d_neg / (d_lower + d_upper)
// (the two planes' distances add up to the cell's width there).  Only steers which exact path
// the learned form takes, so it may be approximate; a degenerate width gives +inf.
__device__ __forceinline__ float beyond_cells(const float (&dv)[6]) {
  float far = 0.f;
  const int lo[3] = {F_LEFT, F_BOTTOM, F_BACK}, hi[3] = {F_RIGHT, F_TOP, F_FRONT};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float dl = dv[lo[a]], dh = dv[hi[a]], width = dl + dh;
    const float neg = dl < 0.f ? -dl : (dh < 0.f ? -dh : 0.f);
    if (neg > 0.f) far = fmaxf(far, width > 0.f ? __fdividef(neg, width) : INFINITY);
  }
  return far;
}

// Advect + locate, one thread per particle.
//   FIRST == false: the reference walk from the previous cell (or cell (0,0,0)).
//   FIRST == true:  the reference's first evaluation, in the previous cell; a particle that it
//                   does not conclude and that lies at least far_cells past that cell is
//                   marked in `pending` (per warp of slots: a bit mask [W] and its count
//                   [W + 1], W = ceil(n_cap / 32)) with its cell field set to P1, the
//                   walk's second cell, and finished by k_locate32_path (its key and
//                   histogram entry are written there); a nearer one continues the reference
//                   walk here.
template <bool FIRST>
__global__ void __launch_bounds__(FDF_LOC_THREADS, FDF_LOC_MIN_BLOCKS) k_locate32(SwarmBuf b, GridDims g, const float *__restrict__ table,
                                                  const double *__restrict__ planes, float dt32, int advect,
                                                  int reset_first, const double *__restrict__ bbox,
                                                  const float *__restrict__ fbox, int drop_removed,
                                                  DevCounters *cnt, unsigned int *__restrict__ keys,
                                                  unsigned int *__restrict__ rank,
                                                  unsigned int *__restrict__ count, unsigned int sentinel,
                                                  unsigned int *__restrict__ pending, int n_cap, float far_cells) {
  const int n = cnt->n_sorted;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0 && advect) atomicAdd(&cnt->psteps_total, (unsigned long long)n);
  LocCounts m;
  unsigned int hkey = 0xffffffffu;
  bool wait = false;
  if (s < n) {
    float2 px = ld_pair(b.x, s), py = ld_pair(b.y, s), pz = ld_pair(b.z, s);
    if (advect) {   // FP32 displacement added to the (hi, lo) position
      px = pair_add(px, __fmul_rn(b.uf[s], dt32));
      py = pair_add(py, __fmul_rn(b.vf[s], dt32));
      pz = pair_add(pz, __fmul_rn(b.wf[s], dt32));
      st_pair(b.x, s, px); st_pair(b.y, s, py); st_pair(b.z, s, pz);
    }
    unsigned char st = b.status[s];
    if (reset_first && st == ST_ACTIVE_AND_LOCATED) st = ST_NEEDS_LOCATION;
    int cell = b.cell[s];
    bool lost = false;
    if (st != ST_ACTIVE_AND_LOCATED) {
      Walk32 w;
      w.i = 0; w.j = 0; w.k = 0; w.err = 0u;
      if (cell >= 0 && (long long)cell < g.Nc) cell_ijk(g, (unsigned int)cell, w.i, w.j, w.k);
      walk_ref32(table, planes, g, px, py, pz, FIRST ? 1 : FDF_MAX_TRAVERSAL, w, m.fb);
      m.err |= w.err;
      m.done += (unsigned int)w.evaluated;
      // learned form: the walk's next cell (w.i, w.j, k) is where the reference continues;
      // outside the grid it ends there as LOST, as the reference's next loop test does
      const bool next_inside = w.i >= 0 && w.i < g.IM && w.j >= 0 && w.j < g.JM && w.k >= 0 && w.k < g.KM;
      if (FIRST && !w.concluded && !w.lost && next_inside && !(far_cells <= beyond_cells(w.e.dv))) {
        // close to the previous cell: the reference walk continues here from its second cell
        Walk32 w2;
        w2.i = w.i; w2.j = w.j; w2.k = w.k; w2.err = 0u;
        walk_ref32(table, planes, g, px, py, pz, FDF_MAX_TRAVERSAL - 1, w2, m.fb);
        m.err |= w2.err;
        m.done += (unsigned int)w2.evaluated;
        m.evals += (unsigned int)(w.evaluated + w2.evaluated);
        lost = w2.lost || !w2.concluded;
        store_located32(b, s, g, lost, w2.i, w2.j, w2.k, w2.e.dv);
        cell = lost ? -1 : (int)(((long long)w2.k * g.JM + w2.j) * g.IM + w2.i);
      } else if (FIRST && !w.concluded && !w.lost && next_inside) {
        wait = true;
        m.evals += (unsigned int)w.evaluated;
        b.cell[s] = (int)(((long long)w.k * g.JM + w.j) * g.IM + w.i);
      } else {
        m.evals += FIRST ? (unsigned int)w.evaluated : (unsigned int)(w.cycle ? FDF_MAX_TRAVERSAL : w.steps);
        lost = w.lost || !w.concluded;
        store_located32(b, s, g, lost, w.i, w.j, w.k, w.e.dv);
        cell = lost ? -1 : (int)(((long long)w.k * g.JM + w.j) * g.IM + w.i);
      }
    } else {
      lost = (cell < 0);
    }
    if (!wait) {
      const unsigned int key =
          settle_key32(lost, cell, px, py, pz, drop_removed, bbox, fbox, sentinel, m.lost, m.oob, m.lost_total);
      keys[s] = key;
      if (key < sentinel) hkey = key;
      else if (!drop_removed) hkey = sentinel;
    }
  }
  if (FIRST) {   // the warp's pending slots as a bit mask and its count (scanned, then compacted)
    const unsigned int mask = __ballot_sync(0xffffffffu, s < n_cap && wait);
    const int W = (n_cap + 31) >> 5, w = s >> 5;
    if ((threadIdx.x & 31) == 0 && w < W) {
      pending[w] = mask;
      pending[W + w] = (unsigned int)__popc(mask);
      if (w == 0) pending[2 * W] = 0u;
    }
  }
  const unsigned int r = warp_histogram_rank(hkey, count);
  if (hkey != 0xffffffffu) rank[s] = r;
  block_flush_counts(m, cnt);
}

// pf = the warps' masks [W], then the exclusive scan of their counts [W + 1]: warp w's pending
// slots go to list[scan[w]...] in ascending order, which keeps the slot (cell) order.
__global__ void k_compact_pending(const unsigned int *__restrict__ pf, int n_cap, unsigned int *__restrict__ list,
                                  DevCounters *cnt) {
  const int W = (n_cap + 31) >> 5;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w == 0) cnt->pending = pf[2 * W];
  if (w < W) {
    unsigned int m = pf[w], o = pf[W + w];
    while (m) {
      list[o++] = (unsigned int)(32 * w + __ffs((int)m) - 1);
      m &= m - 1u;
    }
  }
}

// The pending particles of the learned form (the list from k_locate32<true>; b.cell[s] holds P1,
// the reference walk's second cell): the reference walk from P1, exactly as the FP32 form walks
// it, with the plane-table rows of the path the network predicts -- P1 stepping one index per
// axis toward the guessed cell -- prefetched into L1 ahead of the walk (`lookahead` cells after
// P1).  Whatever the guess, the cells, weights and statuses are the reference walk's; a good
// guess turns the walk's dependent row loads into L1 hits.  Grid-stride over the list with a
// warp-uniform trip count; path_hits counts the evaluations whose row was prefetched.
__device__ __forceinline__ void prefetch_row_l1(const float *row) {   // a row is one 128-B line
  asm volatile("prefetch.global.L1 [%0];" ::"l"(row));
}

__global__ void __launch_bounds__(FDF_GUESS_THREADS, FDF_GUESS_MIN_BLOCKS) k_locate32_path(SwarmBuf b, GridDims g, const float *__restrict__ table,
                                                        const double *__restrict__ planes,
                                                        const double *__restrict__ bbox,
                                                        const float *__restrict__ fbox, int drop_removed,
                                                        DevCounters *cnt, unsigned int *__restrict__ keys,
                                                        unsigned int *__restrict__ rank,
                                                        unsigned int *__restrict__ count, unsigned int sentinel,
                                                        const unsigned int *__restrict__ pending,
                                                        const int *__restrict__ guess, int lookahead) {
  const long long npend = (long long)cnt->pending;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  unsigned int pev = 0, hits = 0;
  LocCounts m;
  for (long long base = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); base < npend; base += stride) {
    const long long t = base + lane;
    unsigned int hkey = 0xffffffffu;
    int s = 0;
    if (t < npend) {
      s = (int)pending[t];
      const float2 px = ld_pair(b.x, s), py = ld_pair(b.y, s), pz = ld_pair(b.z, s);
      Walk32 w;
      w.err = 0u;
      cell_ijk(g, (unsigned int)b.cell[s], w.i, w.j, w.k);
      int gi, gj, gk;
      cell_ijk(g, (unsigned int)guess[t], gi, gj, gk);
      // P1 and the guess lie in the grid, so does every cell of the path between them
      for (int q = 1; q <= lookahead; ++q) {
        const int ci = path_index(w.i, gi, q), cj = path_index(w.j, gj, q), ck = path_index(w.k, gk, q);
        prefetch_row_l1(table + (((long long)ck * g.JM + cj) * g.IM + ci) * FDF_ROW32);
        if (ci == gi && cj == gj && ck == gk) break;   // the predicted path has reached the guess
      }
      walk_ref32<false, true>(table, planes, g, px, py, pz, FDF_MAX_TRAVERSAL - 1, w, m.fb, 0.0, 0.0, 0.0, gi, gj,
                              gk, &hits);
      m.err |= w.err;
      m.done += (unsigned int)w.evaluated;
      m.evals += (unsigned int)w.evaluated;
      pev += (unsigned int)w.evaluated;
      const bool lost = w.lost || !w.concluded;
      store_located32(b, s, g, lost, w.i, w.j, w.k, w.e.dv);
      const int cell = lost ? -1 : (int)(((long long)w.k * g.JM + w.j) * g.IM + w.i);
      const unsigned int key =
          settle_key32(lost, cell, px, py, pz, drop_removed, bbox, fbox, sentinel, m.lost, m.oob, m.lost_total);
      keys[s] = key;
      if (key < sentinel) hkey = key;
      else if (!drop_removed) hkey = sentinel;
    }
    const unsigned int r = warp_histogram_rank(hkey, count);
    if (hkey != 0xffffffffu) rank[s] = r;
  }
  block_flush_counts(m, cnt);
  block_add_u64(hits, &cnt->guess_taken_total);
  block_add_u64(pev, &cnt->guess_evals_total);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->guess_asked_total, (unsigned long long)npend);
}

// UpdateAllParticlePositions in the precision form: fl32(v dt) added to the (hi, lo) position,
// as the fused step does it.
__global__ void k_advect32(SwarmBuf b, float dt32, DevCounters *cnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) atomicAdd(&cnt->psteps_total, (unsigned long long)cnt->n_sorted);   // particles advanced
  if (s >= cnt->n_sorted) return;
  st_pair(b.x, s, pair_add(ld_pair(b.x, s), __fmul_rn(b.uf[s], dt32)));
  st_pair(b.y, s, pair_add(ld_pair(b.y, s), __fmul_rn(b.vf[s], dt32)));
  st_pair(b.z, s, pair_add(ld_pair(b.z, s), __fmul_rn(b.wf[s], dt32)));
}

// Sort keys of the particles held (a re-sort by cell), dropping the LOST ones
// (CheckAndRemoveLostParticles, ParticleMotion.c:532-625) and/or the ones outside the
// bounding box (CheckAndRemoveOutOfBoundsParticles, :283-383; the FP32 form decides as the
// step does).  Kept particles without a cell go to the LOST bucket at the end; the removed
// ones get key all ones and no slot.
template <bool F32>
__global__ void __launch_bounds__(256) k_resort_keys(SwarmBuf b, GridDims g, int remove_lost, int remove_oob,
                                                    const double *__restrict__ bbox, const float *__restrict__ fbox,
                                                    DevCounters *cnt, unsigned int *__restrict__ keys,
                                                    unsigned int *__restrict__ rank, unsigned int *__restrict__ count,
                                                    unsigned int sentinel) {
  const int n = cnt->n_sorted;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  LocCounts m;
  unsigned int hkey = 0xffffffffu;
  if (s < n) {
    const int cell = b.cell[s];
    unsigned int key = (cell >= 0 && (long long)cell < g.Nc) ? (unsigned int)cell : sentinel;
    if (remove_lost && b.status[s] == ST_LOST) {
      m.lost += 1;
      key = 0xffffffffu;
    } else if (remove_oob) {
      bool inside;
      if (F32) {
        const float2 px = ld_pair(b.x, s), py = ld_pair(b.y, s), pz = ld_pair(b.z, s);
        unsigned int l0 = 0, o1 = 0, l2 = 0;
        inside = settle_key32(false, 0, px, py, pz, 1, bbox, fbox, sentinel, l0, o1, l2) != sentinel;
      } else {
        const double x = b.x[s], y = b.y[s], z = b.z[s];
        inside = x >= bbox[0] && x <= bbox[3] && y >= bbox[1] && y <= bbox[4] && z >= bbox[2] && z <= bbox[5];
      }
      if (!inside) {
        m.oob += 1;
        key = 0xffffffffu;
      }
    }
    keys[s] = key;
    hkey = key;
  }
  const unsigned int r = warp_histogram_rank(hkey, count);
  if (hkey != 0xffffffffu) rank[s] = r;
  block_flush_counts(m, cnt);
}

// Corner field in FP32: mean of the valid adjacent cells (nodes next to occupied cells).
__global__ void k_center_to_corner32(const float *__restrict__ ucat, GridDims g, float *__restrict__ corner,
                                     const unsigned int *__restrict__ cell_start, unsigned long long *nodes_done) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool work = q < g.Nn;
  int i = 0, j = 0, k = 0;
  if (work) node_ijk(g, (unsigned int)q, i, j, k);
  if (cell_start) {
    bool need = false;
    if (work)
      for (int dk = -1; dk <= 0 && !need; ++dk)
        for (int dj = -1; dj <= 0 && !need; ++dj)
          for (int di = -1; di <= 0 && !need; ++di) {
            int ck = k + dk, cj = j + dj, ci = i + di;
            if (ci < 0 || ci >= g.IM || cj < 0 || cj >= g.JM || ck < 0 || ck >= g.KM) continue;
            long long c = ((long long)ck * g.JM + cj) * g.IM + ci;
            need = __ldg(cell_start + c + 1) > __ldg(cell_start + c);
          }
    if (nodes_done) block_add_u64(need ? 1ull : 0ull, nodes_done);
    if (!need) return;
  }
  if (!work) return;
  float sx = 0.f, sy = 0.f, sz = 0.f;
  int count = 0;
#pragma unroll
  for (int dk = -1; dk <= 0; ++dk)
#pragma unroll
    for (int dj = -1; dj <= 0; ++dj)
#pragma unroll
      for (int di = -1; di <= 0; ++di) {
        const int ck = k + dk, cj = j + dj, ci = i + di;
        if (ci < 0 || ci >= g.IM || cj < 0 || cj >= g.JM || ck < 0 || ck >= g.KM) continue;
        const long long c = ((long long)ck * g.JM + cj) * g.IM + ci;
        sx += __ldg(ucat + c); sy += __ldg(ucat + g.Nc + c); sz += __ldg(ucat + 2 * g.Nc + c);
        ++count;
      }
  const float r = count == 8 ? 0.125f : count == 4 ? 0.25f : count == 2 ? 0.5f : count == 1 ? 1.0f : 0.0f;
  corner[q] = sx * r; corner[g.Nn + q] = sy * r; corner[2 * g.Nn + q] = sz * r;
}

__global__ void __launch_bounds__(256) k_gather_interp32(SwarmBuf src, SwarmBuf dst, GridDims g,
                                                         const float *__restrict__ corner,
                                                         const unsigned int *__restrict__ perm,
                                                         const unsigned int *__restrict__ cell_start,
                                                         DevCounters *cnt, int mode) {
  const int n = (int)cell_start[g.Nc + 1];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    cnt->n = (int)cell_start[g.Nc];
    cnt->n_sorted = n;
  }
  if (s >= n) return;
  const unsigned int p = perm ? perm[s] : (unsigned int)s;
  const int cell = src.cell[p];
  float a1 = src.a1f[p], a2 = src.a2f[p], a3 = src.a3f[p];
  const unsigned char st = src.status[p];
  dst.x[s] = src.x[p]; dst.y[s] = src.y[p]; dst.z[s] = src.z[p];
  dst.a1f[s] = a1; dst.a2f[s] = a2; dst.a3f[s] = a3;
  dst.Pf[s] = src.Pf[p];
  dst.pid[s] = src.pid[p];
  if (mode == GATHER_COPY) {
    dst.uf[s] = src.uf[p]; dst.vf[s] = src.vf[p]; dst.wf[s] = src.wf[p];
    dst.cell[s] = cell;
    dst.status[s] = st;
    return;
  }
  float ux = 0.f, uy = 0.f, uz = 0.f;
  if (cell < 0) {
    dst.cell[s] = -1;
    dst.status[s] = mode == GATHER_INTERP ? (unsigned char)ST_LOST : st;
  } else {
    dst.cell[s] = cell;
    dst.status[s] = mode == GATHER_INTERP ? (unsigned char)ST_ACTIVE_AND_LOCATED : st;
    int i, j, k;
    cell_ijk(g, (unsigned int)cell, i, j, k);
    a1 = fminf(fmaxf(a1, 0.f), 1.f);   // NaN -> 0 as PetscMax(0, PetscMin(1, NaN))
    a2 = fminf(fmaxf(a2, 0.f), 1.f);
    a3 = fminf(fmaxf(a3, 0.f), 1.f);
    const float oa1 = 1.f - a1, oa2 = 1.f - a2, oa3 = 1.f - a3;
    const float p00 = oa1 * oa2, p10 = a1 * oa2, p01 = oa1 * a2, p11 = a1 * a2;
    const float w[8] = {p00 * oa3, p10 * oa3, p01 * oa3, p11 * oa3, p00 * a3, p10 * a3, p01 * a3, p11 * a3};
    const long long mx = g.IM + 1, my = g.JM + 1;
    const long long q0 = ((long long)k * my + j) * mx + i;
    const long long off[8] = {0, 1, mx, mx + 1, mx * my, mx * my + 1, mx * my + mx, mx * my + mx + 1};
    float sw = 0.f, ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const long long q = q0 + off[c];
      ax = fmaf(w[c], __ldg(corner + q), ax);
      ay = fmaf(w[c], __ldg(corner + g.Nn + q), ay);
      az = fmaf(w[c], __ldg(corner + 2 * g.Nn + q), az);
      sw += w[c];
    }
    if (sw > 1.0e-14f) { ux = ax / sw; uy = ay / sw; uz = az / sw; }
  }
  dst.uf[s] = ux; dst.vf[s] = uy; dst.wf[s] = uz;
}

// Neumaier-compensated running sum.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float t = s + v;
    if (fabsf(s) >= fabsf(v)) c += (s - t) + v; else c += (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

// Resident 256-thread blocks per SM the volume and the momentum deposits are compiled for.  The
// per-node chains wait on their loads, so 2048 resident threads (32 registers, a few spilled)
// beat the 48-register default for the volume deposit: 0.617 -> 0.532 ms per 64M-particle step
// (0.558 at 5 blocks, 0.550 at 6); 1024 (64 registers) beat 768 (80) for the momentum deposit:
// 2.95 -> 2.88 ms per 128M-particle step.
#ifndef FDF_DEP32_MIN_BLOCKS
#define FDF_DEP32_MIN_BLOCKS 8
#endif
#ifndef FDF_DEPM32_MIN_BLOCKS
#define FDF_DEPM32_MIN_BLOCKS 4
#endif
template <bool MOM>
__global__ void __launch_bounds__(256, MOM ? FDF_DEPM32_MIN_BLOCKS : FDF_DEP32_MIN_BLOCKS) k_deposit32(SwarmBuf b, GridDims g, const unsigned int *__restrict__ cs,
                                                   float third, float *__restrict__ count, float *__restrict__ avg,
                                                   float *__restrict__ fi, float *__restrict__ fj,
                                                   float *__restrict__ fk, float *__restrict__ mi,
                                                   float *__restrict__ mj, float *__restrict__ mk) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nn) return;
  const int IM = g.IM, JM = g.JM, KM = g.KM;
  int i, j, k;
  node_ijk(g, (unsigned int)q, i, j, k);
  const bool is_cell = i < IM && j < JM && k < KM;
  const long long c = ((long long)k * JM + j) * IM + i;
  int s0 = 0, s1 = 0;
  if (is_cell) { s0 = (int)__ldg(cs + c); s1 = (int)__ldg(cs + c + 1); }
  // per face the lower cell's segment first, then this cell's; the three lower segments run
  // first and this cell's segment then feeds the P sum and the three upper parts in one pass
  // (every accumulator receives its values in the same order as face by face)
  const long long nfi = (IM + 1LL) * JM * KM, nfj = IM * (JM + 1LL) * KM, nfk = (long long)IM * JM * (KM + 1LL);
  const bool face_i = j < JM && k < KM, face_j = i < IM && k < KM, face_k = i < IM && j < JM;
  KSum acc[3], mm[3][3];
  // Each segment is read in chunks of DCH particles, all loads of a chunk issued before its
  // in-order adds, so one load latency serves the chunk instead of each particle.
  constexpr int DCH = MOM ? 4 : 8;
  auto lower = [&](int f, const float *__restrict__ wgt, long long lc) {
    const int l0 = (int)__ldg(cs + lc), l1 = (int)__ldg(cs + lc + 1);
    for (int s = l0; s < l1; s += DCH) {
      float a[DCH], u[DCH], v[DCH], w[DCH];
#pragma unroll
      for (int q = 0; q < DCH; ++q) {
        const bool in = s + q < l1;
        a[q] = in ? __ldg(wgt + s + q) : 0.f;
        if (MOM) {
          u[q] = in ? __ldg(b.uf + s + q) : 0.f;
          v[q] = in ? __ldg(b.vf + s + q) : 0.f;
          w[q] = in ? __ldg(b.wf + s + q) : 0.f;
        }
      }
#pragma unroll
      for (int q = 0; q < DCH; ++q) {
        if (s + q >= l1) break;
        const float fr = a[q] * third;
        acc[f].add(fr);
        if (MOM) { mm[f][0].add(fr * u[q]); mm[f][1].add(fr * v[q]); mm[f][2].add(fr * w[q]); }
      }
    }
  };
  if (face_i && i > 0) lower(0, b.a1f, c - 1);
  if (face_j && j > 0) lower(1, b.a2f, ((long long)k * JM + (j - 1)) * IM + i);
  if (face_k && k > 0) lower(2, b.a3f, ((long long)(k - 1) * JM + j) * IM + i);
  KSum sum;
  constexpr int OCH = 4;
  for (int s = s0; s < s1; s += OCH) {
    float P[OCH], w[OCH][3], u[OCH], v[OCH], ww[OCH];
#pragma unroll
    for (int q = 0; q < OCH; ++q) {
      const bool in = s + q < s1;
      P[q] = in ? __ldg(b.Pf + s + q) : 0.f;
      w[q][0] = in ? __ldg(b.a1f + s + q) : 0.f;
      w[q][1] = in ? __ldg(b.a2f + s + q) : 0.f;
      w[q][2] = in ? __ldg(b.a3f + s + q) : 0.f;
      if (MOM) {
        u[q] = in ? __ldg(b.uf + s + q) : 0.f;
        v[q] = in ? __ldg(b.vf + s + q) : 0.f;
        ww[q] = in ? __ldg(b.wf + s + q) : 0.f;
      }
    }
#pragma unroll
    for (int q = 0; q < OCH; ++q) {
      if (s + q >= s1) break;
      sum.add(P[q]);
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const float fr = (1.f - w[q][f]) * third;
        acc[f].add(fr);
        if (MOM) { mm[f][0].add(fr * u[q]); mm[f][1].add(fr * v[q]); mm[f][2].add(fr * ww[q]); }
      }
    }
  }
  {
    const int nc = s1 - s0;
    count[q] = (float)nc;
    avg[q] = nc > 0 ? sum.value() / (float)nc : 0.f;
  }
  auto store = [&](int f, float *vol, float *mom, long long nf, long long fidx) {
    vol[fidx] = acc[f].value();
    if (MOM) { mom[fidx] = mm[f][0].value(); mom[nf + fidx] = mm[f][1].value(); mom[2 * nf + fidx] = mm[f][2].value(); }
  };
  if (face_i) store(0, fi, mi, nfi, ((long long)k * JM + j) * (IM + 1) + i);
  if (face_j) store(1, fj, mj, nfj, ((long long)k * (JM + 1) + j) * IM + i);
  if (face_k) store(2, fk, mk, nfk, c);
}

__global__ void k_from_aos32(const double *__restrict__ pos, const double *__restrict__ vel,
                             const double *__restrict__ wgt, const double *__restrict__ P,
                             const long long *__restrict__ cell3, const long long *__restrict__ pid,
                             const long long *__restrict__ status, int n, GridDims g, SwarmBuf b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  for (int q = 0; q < 3; ++q) {
    const double v = pos[3 * p + q];
    const float h = __double2float_rn(v);
    const float l = __double2float_rn(__dsub_rn(v, (double)h));
    st_pair(q == 0 ? b.x : q == 1 ? b.y : b.z, p, make_float2(h, l));
  }
  b.uf[p] = (float)vel[3 * p]; b.vf[p] = (float)vel[3 * p + 1]; b.wf[p] = (float)vel[3 * p + 2];
  b.a1f[p] = (float)wgt[3 * p]; b.a2f[p] = (float)wgt[3 * p + 1]; b.a3f[p] = (float)wgt[3 * p + 2];
  b.Pf[p] = (float)P[p];
  b.pid[p] = pid[p];
  const long long i = cell3[3 * p], j = cell3[3 * p + 1], k = cell3[3 * p + 2];
  int c = -1;
  if (i >= 0 && i < g.IM && j >= 0 && j < g.JM && k >= 0 && k < g.KM) c = (int)((k * g.JM + j) * g.IM + i);
  b.cell[p] = c;
  const long long st = status[p];
  b.status[p] = (unsigned char)((st >= 0 && st <= ST_UNINITIALIZED) ? st : ST_UNINITIALIZED);
}

__global__ void k_to_aos32(SwarmBuf b, int n, GridDims g, double *__restrict__ pos, double *__restrict__ vel,
                           double *__restrict__ wgt, double *__restrict__ P, long long *__restrict__ cell3,
                           long long *__restrict__ pid, long long *__restrict__ status) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  pos[3 * p] = pair_value(ld_pair(b.x, p));
  pos[3 * p + 1] = pair_value(ld_pair(b.y, p));
  pos[3 * p + 2] = pair_value(ld_pair(b.z, p));
  vel[3 * p] = b.uf[p]; vel[3 * p + 1] = b.vf[p]; vel[3 * p + 2] = b.wf[p];
  wgt[3 * p] = b.a1f[p]; wgt[3 * p + 1] = b.a2f[p]; wgt[3 * p + 2] = b.a3f[p];
  P[p] = b.Pf[p];
  pid[p] = b.pid[p];
  const int c = b.cell[p];
  if (c >= 0) {
    int i, j, k;
    cell_ijk(g, (unsigned int)c, i, j, k);
    cell3[3 * p] = i; cell3[3 * p + 1] = j; cell3[3 * p + 2] = k;
  } else {
    cell3[3 * p] = -1; cell3[3 * p + 1] = -1; cell3[3 * p + 2] = -1;
  }
  status[p] = b.status[p];
}

// Layout conversion straight from / to the caller's page-locked DMSwarm arrays over the host
// link.  A block stages 256 particles' AoS records (15 x 8 B each: position, velocity, weights,
// P, cell triple, PID, status) in shared memory, moving each field's contiguous range with
// coalesced 16-byte accesses -- the access pattern that reaches the link's copy rate -- and each
// thread converts its own particle to or from the device SoA buffers as the per-particle
// kernels above do.  The arrays must be 16-byte aligned.
constexpr int XF_TILE = 256;
// field f: doubles per particle, and the field's offset in the shared tile (in doubles)
__host__ __device__ constexpr int xf_bs(int f) { return (f < 3 || f == 4) ? 3 : 1; }
__host__ __device__ constexpr int xf_off(int f) { return XF_TILE * (f <= 3 ? 3 * f : f == 4 ? 10 : f == 5 ? 13 : 14); }

struct HostSwarm {
  const double *f[7];   // position, velocity, weight, P, cell (int64), pid (int64), status (int64)
};

__device__ __forceinline__ void tile_in(double *dst, const double *__restrict__ src, int count) {
  const double2 *s2 = reinterpret_cast<const double2 *>(src);
  double2 *d2 = reinterpret_cast<double2 *>(dst);
  for (int q = threadIdx.x; q < count / 2; q += XF_TILE) d2[q] = s2[q];
  if ((count & 1) && threadIdx.x == 0) dst[count - 1] = src[count - 1];
}
__device__ __forceinline__ void tile_out(double *__restrict__ dst, const double *src, int count) {
  const double2 *s2 = reinterpret_cast<const double2 *>(src);
  double2 *d2 = reinterpret_cast<double2 *>(dst);
  for (int q = threadIdx.x; q < count / 2; q += XF_TILE) d2[q] = s2[q];
  if ((count & 1) && threadIdx.x == 0) dst[count - 1] = src[count - 1];
}

template <bool F32>
__global__ void __launch_bounds__(XF_TILE) k_from_host(HostSwarm h, int n, GridDims g, SwarmBuf b) {
  __shared__ __align__(16) double sm[15 * XF_TILE];
  const int p0 = blockIdx.x * XF_TILE, m = min(XF_TILE, n - p0);
#pragma unroll
  for (int f = 0; f < 7; ++f) tile_in(sm + xf_off(f), h.f[f] + (long long)xf_bs(f) * p0, xf_bs(f) * m);
  __syncthreads();
  const int t = threadIdx.x;
  if (t >= m) return;
  const int p = p0 + t;
  const double *pos = sm + xf_off(0) + 3 * t, *vel = sm + xf_off(1) + 3 * t, *wgt = sm + xf_off(2) + 3 * t;
  const long long *c3 = reinterpret_cast<const long long *>(sm + xf_off(4)) + 3 * t;
  if (F32) {
    st_pair(b.x, p, fdfx::split_rn(pos[0])); st_pair(b.y, p, fdfx::split_rn(pos[1])); st_pair(b.z, p, fdfx::split_rn(pos[2]));
    b.uf[p] = fdfx::d2f_rn(vel[0]); b.vf[p] = fdfx::d2f_rn(vel[1]); b.wf[p] = fdfx::d2f_rn(vel[2]);
    b.a1f[p] = fdfx::d2f_rn(wgt[0]); b.a2f[p] = fdfx::d2f_rn(wgt[1]); b.a3f[p] = fdfx::d2f_rn(wgt[2]);
    b.Pf[p] = fdfx::d2f_rn(sm[xf_off(3) + t]);
  } else {
    b.x[p] = pos[0]; b.y[p] = pos[1]; b.z[p] = pos[2];
    b.u[p] = vel[0]; b.v[p] = vel[1]; b.w[p] = vel[2];
    b.a1[p] = wgt[0]; b.a2[p] = wgt[1]; b.a3[p] = wgt[2];
    b.P[p] = sm[xf_off(3) + t];
  }
  b.pid[p] = reinterpret_cast<const long long *>(sm + xf_off(5))[t];
  const long long i = c3[0], j = c3[1], k = c3[2];
  int c = -1;
  if (i >= 0 && i < g.IM && j >= 0 && j < g.JM && k >= 0 && k < g.KM) c = (int)((k * g.JM + j) * g.IM + i);
  b.cell[p] = c;
  const long long st = reinterpret_cast<const long long *>(sm + xf_off(6))[t];
  b.status[p] = (unsigned char)((st >= 0 && st <= ST_UNINITIALIZED) ? st : ST_UNINITIALIZED);
}

template <bool F32>
__global__ void __launch_bounds__(XF_TILE) k_to_host(SwarmBuf b, int n, GridDims g, HostSwarm h) {
  __shared__ __align__(16) double sm[15 * XF_TILE];
  const int p0 = blockIdx.x * XF_TILE, m = min(XF_TILE, n - p0);
  const int t = threadIdx.x;
  if (t < m) {
    const int p = p0 + t;
    double *pos = sm + xf_off(0) + 3 * t, *vel = sm + xf_off(1) + 3 * t, *wgt = sm + xf_off(2) + 3 * t;
    if (F32) {
      pos[0] = pair_value(ld_pair(b.x, p)); pos[1] = pair_value(ld_pair(b.y, p)); pos[2] = pair_value(ld_pair(b.z, p));
      vel[0] = b.uf[p]; vel[1] = b.vf[p]; vel[2] = b.wf[p];
      wgt[0] = b.a1f[p]; wgt[1] = b.a2f[p]; wgt[2] = b.a3f[p];
      sm[xf_off(3) + t] = b.Pf[p];
    } else {
      pos[0] = b.x[p]; pos[1] = b.y[p]; pos[2] = b.z[p];
      vel[0] = b.u[p]; vel[1] = b.v[p]; vel[2] = b.w[p];
      wgt[0] = b.a1[p]; wgt[1] = b.a2[p]; wgt[2] = b.a3[p];
      sm[xf_off(3) + t] = b.P[p];
    }
    long long *c3 = reinterpret_cast<long long *>(sm + xf_off(4)) + 3 * t;
    const int c = b.cell[p];
    if (c >= 0) {
      int i, j, k;
      cell_ijk(g, (unsigned int)c, i, j, k);
      c3[0] = i; c3[1] = j; c3[2] = k;
    } else {
      c3[0] = -1; c3[1] = -1; c3[2] = -1;
    }
    reinterpret_cast<long long *>(sm + xf_off(5))[t] = b.pid[p];
    reinterpret_cast<long long *>(sm + xf_off(6))[t] = b.status[p];
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < 7; ++f)
    tile_out(const_cast<double *>(h.f[f]) + (long long)xf_bs(f) * p0, sm + xf_off(f), xf_bs(f) * m);
}

__global__ void k_f64_to_f32(const double *__restrict__ in, float *__restrict__ out, long long n) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) out[q] = (float)in[q];
}

__global__ void k_f32_to_f64(const float *__restrict__ in, double *__restrict__ out, long long n) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) out[q] = (double)in[q];
}

inline unsigned int blocks_for(long long n, int th) { return (unsigned int)(n > 0 ? (n + th - 1) / th : 1); }

}  // namespace

void launch_build_table32(const double *planes, const double *coor, GridDims g, float *table, cudaStream_t s) {
  k_build_table32<<<blocks_for(g.Nc, 128), 128, 0, s>>>(planes, coor, g, table);
}

void launch_locate32(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes, double dt,
                     int advect, const double *bbox, const float *fbox, int drop_removed, DevCounters *cnt,
                     unsigned int *keys, unsigned int *rank, unsigned int *count, unsigned int sentinel,
                     unsigned int *pending, float far_cells, cudaStream_t s) {
  constexpr int th = FDF_LOC_THREADS;
  if (pending)
    k_locate32<true><<<blocks_for(n_cap, th), th, 0, s>>>(b, g, table, planes, (float)dt, advect, drop_removed, bbox,
                                                          fbox, drop_removed, cnt, keys, rank, count, sentinel,
                                                          pending, n_cap, far_cells);
  else
    k_locate32<false><<<blocks_for(n_cap, th), th, 0, s>>>(b, g, table, planes, (float)dt, advect, drop_removed,
                                                           bbox, fbox, drop_removed, cnt, keys, rank, count, sentinel,
                                                           nullptr, n_cap, 0.f);
}

void launch_compact_pending(const unsigned int *scan, int n_cap, unsigned int *list, DevCounters *cnt,
                            cudaStream_t s) {
  k_compact_pending<<<blocks_for((n_cap + 31) / 32, 256), 256, 0, s>>>(scan, n_cap, list, cnt);
}

void launch_locate32_path(const SwarmBuf &b, int n_cap, GridDims g, const float *table, const double *planes,
                          const double *bbox, const float *fbox, int drop_removed, DevCounters *cnt,
                          unsigned int *keys, unsigned int *rank, unsigned int *count, unsigned int sentinel,
                          const unsigned int *pending, const int *guess, int num_sms, cudaStream_t s) {
  // grid-stride kernel: one wave of resident blocks, so that no SM runs a partial last wave
  static int resident = 0, res_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (res_device != dev) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_locate32_path, FDF_GUESS_THREADS, 0);
    res_device = dev;
  }
  const long long need = ((long long)n_cap + FDF_GUESS_THREADS - 1) / FDF_GUESS_THREADS;
  long long blocks = (long long)num_sms * (resident > 0 ? resident : 1);
  if (blocks > need) blocks = need;
  k_locate32_path<<<(unsigned)(blocks < 1 ? 1 : blocks), FDF_GUESS_THREADS, 0, s>>>(
      b, g, table, planes, bbox, fbox, drop_removed, cnt, keys, rank, count, sentinel, pending, guess,
      FDF_PATH_LOOKAHEAD);
}

void launch_center_to_corner32(const float *ucat, GridDims g, float *corner, const unsigned int *cell_start,
                               unsigned long long *nodes_done, cudaStream_t s) {
  k_center_to_corner32<<<blocks_for(g.Nn, 256), 256, 0, s>>>(ucat, g, corner, cell_start, nodes_done);
}

void launch_advect32(const SwarmBuf &b, int n_cap, double dt, DevCounters *cnt, cudaStream_t s) {
  k_advect32<<<blocks_for(n_cap, 256), 256, 0, s>>>(b, (float)dt, cnt);
}

void launch_resort_keys(const SwarmBuf &b, int n_cap, GridDims g, int f32, int remove_lost, int remove_oob,
                        const double *bbox, const float *fbox, DevCounters *cnt, unsigned int *keys,
                        unsigned int *rank, unsigned int *count, unsigned int sentinel, cudaStream_t s) {
  if (f32)
    k_resort_keys<true><<<blocks_for(n_cap, 256), 256, 0, s>>>(b, g, remove_lost, remove_oob, bbox, fbox, cnt, keys,
                                                               rank, count, sentinel);
  else
    k_resort_keys<false><<<blocks_for(n_cap, 256), 256, 0, s>>>(b, g, remove_lost, remove_oob, bbox, fbox, cnt, keys,
                                                                rank, count, sentinel);
}

void launch_gather_interp32(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g, const float *corner,
                            const unsigned int *perm, const unsigned int *cell_start, DevCounters *cnt,
                            cudaStream_t s, int mode) {
  k_gather_interp32<<<blocks_for(n_cap, 256), 256, 0, s>>>(src, dst, g, corner, perm, cell_start, cnt, mode);
}

void launch_deposit32(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, double volume, float *count,
                      float *avg, float *fi, float *fj, float *fk, float *mi, float *mj, float *mk, cudaStream_t s) {
  if (mi)
    k_deposit32<true><<<blocks_for(g.Nn, 256), 256, 0, s>>>(b, g, cell_start, (float)(volume / 3.0), count, avg, fi,
                                                            fj, fk, mi, mj, mk);
  else
    k_deposit32<false><<<blocks_for(g.Nn, 256), 256, 0, s>>>(b, g, cell_start, (float)(volume / 3.0), count, avg, fi,
                                                             fj, fk, nullptr, nullptr, nullptr);
}

void launch_swarm_from_aos32(const double *pos, const double *vel, const double *wgt, const double *P,
                             const long long *cell3, const long long *pid, const long long *status, int n, GridDims g,
                             const SwarmBuf &b, cudaStream_t s) {
  if (n <= 0) return;
  k_from_aos32<<<blocks_for(n, 256), 256, 0, s>>>(pos, vel, wgt, P, cell3, pid, status, n, g, b);
}

void launch_swarm_to_aos32(const SwarmBuf &b, int n, GridDims g, double *pos, double *vel, double *wgt, double *P,
                           long long *cell3, long long *pid, long long *status, cudaStream_t s) {
  if (n <= 0) return;
  k_to_aos32<<<blocks_for(n, 256), 256, 0, s>>>(b, n, g, pos, vel, wgt, P, cell3, pid, status);
}

void launch_swarm_from_host(const void *const f[7], int n, GridDims g, const SwarmBuf &b, bool f32, cudaStream_t s) {
  if (n <= 0) return;
  HostSwarm h;
  for (int q = 0; q < 7; ++q) h.f[q] = static_cast<const double *>(f[q]);
  const unsigned blocks = (unsigned)((n + XF_TILE - 1) / XF_TILE);
  if (f32) k_from_host<true><<<blocks, XF_TILE, 0, s>>>(h, n, g, b);
  else k_from_host<false><<<blocks, XF_TILE, 0, s>>>(h, n, g, b);
}

void launch_swarm_to_host(const SwarmBuf &b, int n, GridDims g, void *const f[7], bool f32, cudaStream_t s) {
  if (n <= 0) return;
  HostSwarm h;
  for (int q = 0; q < 7; ++q) h.f[q] = static_cast<const double *>(f[q]);
  const unsigned blocks = (unsigned)((n + XF_TILE - 1) / XF_TILE);
  if (f32) k_to_host<true><<<blocks, XF_TILE, 0, s>>>(b, n, g, h);
  else k_to_host<false><<<blocks, XF_TILE, 0, s>>>(b, n, g, h);
}

void launch_f64_to_f32(const double *in, float *out, long long n, cudaStream_t s) {
  k_f64_to_f32<<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
}

void launch_f32_to_f64(const float *in, double *out, long long n, cudaStream_t s) {
  k_f32_to_f64<<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
}
