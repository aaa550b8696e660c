// fdf_particles.cu -- grid-to-particle interpolation fused with the sorted
// gather, the deterministic particle-to-grid deposits, and the DMSwarm AoS <->
// device SoA marshalling.
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"

namespace {

using fdfx::add;
using fdfx::sub;
using fdfx::mul;

// Sorted slot s takes the particle from slot perm[s] of the previous order, then
// interpolates ucat to it: ComputeTrilinearWeights (interpolation.c:839-864) and
// TrilinearInterpolation_Vector (:957-1042) from the node-averaged field, with
// the stencil guard of InterpolateEulerFieldToSwarm (:1356-1372).
__global__ void __launch_bounds__(256) k_gather_interp(SwarmBuf src, SwarmBuf dst, GridDims g,
                                                       const double *__restrict__ corner,
                                                       const unsigned int *__restrict__ perm,
                                                       const unsigned int *__restrict__ cell_start,
                                                       DevCounters *cnt, int mode) {
  const int n = (int)cell_start[g.Nc + 1];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {   // the new sizes, read by the next step
    cnt->n = (int)cell_start[g.Nc];
    cnt->n_sorted = n;
  }
  if (s >= n) return;
  const unsigned int p = perm ? perm[s] : (unsigned int)s;
  const int cell = src.cell[p];
  double a1 = src.a1[p], a2 = src.a2[p], a3 = src.a3[p];
  const unsigned char st = src.status[p];
  dst.x[s] = src.x[p]; dst.y[s] = src.y[p]; dst.z[s] = src.z[p];
  dst.a1[s] = a1; dst.a2[s] = a2; dst.a3[s] = a3;
  dst.P[s] = src.P[p];
  dst.pid[s] = src.pid[p];
  if (mode == GATHER_COPY) {
    dst.u[s] = src.u[p]; dst.v[s] = src.v[p]; dst.w[s] = src.w[p];
    dst.cell[s] = cell;
    dst.status[s] = st;
    return;
  }
  double ux = 0.0, uy = 0.0, uz = 0.0;
  if (cell < 0) {
    dst.cell[s] = -1;
    dst.status[s] = mode == GATHER_INTERP ? (unsigned char)ST_LOST : st;
  } else {
    dst.cell[s] = cell;
    dst.status[s] = mode == GATHER_INTERP ? (unsigned char)ST_ACTIVE_AND_LOCATED : st;
    int i, j, k;
    cell_ijk(g, (unsigned int)cell, i, j, k);
    a1 = fdfx::clamp01(a1);
    a2 = fdfx::clamp01(a2);
    a3 = fdfx::clamp01(a3);
    const double oa1 = sub(1.0, a1), oa2 = sub(1.0, a2), oa3 = sub(1.0, a3);
    // w[c] = (x*y)*z as the reference evaluates it; the four (x*y) pair products are shared
    // The 36 products run on the integer pipe (fdfx::mul_int, the same bits as the FP64
    // multiply) and the sums on the FP64 pipe, so both pipes work at once: 8.87 -> 7.78 ms per
    // 64M-particle step against all on the FP64 pipe.
    auto wmul = [](double x, double y) { return fdfx::mul_int(x, y); };
    auto cmul = wmul;
    const double p00 = wmul(oa1, oa2), p10 = wmul(a1, oa2), p01 = wmul(oa1, a2), p11 = wmul(a1, a2);
    double w[8];
    w[0] = wmul(p00, oa3); w[1] = wmul(p10, oa3); w[2] = wmul(p01, oa3); w[3] = wmul(p11, oa3);
    w[4] = wmul(p00, a3);  w[5] = wmul(p10, a3);  w[6] = wmul(p01, a3);  w[7] = wmul(p11, a3);
    const long long mx = g.IM + 1, my = g.JM + 1;
    const long long q0 = ((long long)k * my + j) * mx + i;
    const long long off[8] = {0, 1, mx, mx + 1, mx * my, mx * my + 1, mx * my + mx, mx * my + mx + 1};
    const double *cx = corner, *cy = corner + g.Nn, *cz = corner + 2 * g.Nn;
    // accumulators start at 0.0: the first "0.0 + t" is t except that -0.0 becomes +0.0
    double ax = fdfx::add0(cmul(w[0], __ldg(cx + q0)));
    double ay = fdfx::add0(cmul(w[0], __ldg(cy + q0)));
    double az = fdfx::add0(cmul(w[0], __ldg(cz + q0)));
    double sw = fdfx::add0(w[0]);
#pragma unroll
    for (int c = 1; c < 8; ++c) {
      const long long q = q0 + off[c];
      ax = add(ax, cmul(w[c], __ldg(cx + q)));
      ay = add(ay, cmul(w[c], __ldg(cy + q)));
      az = add(az, cmul(w[c], __ldg(cz + q)));
      sw = add(sw, w[c]);
    }
    // sumW > 1e-14 (false for NaN); x / 1.0 == x exactly, so the common sumW == 1 skips the divides
    if (!fdfx::is_nan(sw) && !fdfx::le_pos(sw, fdfx::ubits(1.0e-14))) {
      if (fdfx::ubits(sw) == 0x3ff0000000000000ULL) {
        ux = ax; uy = ay; uz = az;
      } else {
        const fdfx::Divisor dsw = fdfx::make_divisor(sw);
        ux = fdfx::div_by(ax, dsw); uy = fdfx::div_by(ay, dsw); uz = fdfx::div_by(az, dsw);
      }
    }
  }
  dst.u[s] = ux; dst.v[s] = uy; dst.w[s] = uz;
}

// One thread per grid node (i<=IM, j<=JM, k<=KM).  The node-sized outputs are the
// reference's ParticleCount and P average (interpolation.c:2063-2116): cell (i,j,k)
// sits at node slot (i,j,k).  The thread also owns the three faces whose lower
// corner is this node: i-face (i,j,k) between cells i-1 and i, and likewise j, k.
// A face sums its lower cell's particles (weight a) and then its upper cell's
// (weight 1-a), each in sorted order: a fixed order, so the sum is deterministic.
// The momentum variant adds the same split of V * velocity (SoA [3][faces]), each component
// summed in the same order.
//
// The products are moved out of the per-node loops.  A node's four segment loops have
// different lengths across a warp, and a warp-wide FP64 instruction costs the same with one
// active lane as with 32; so the warp's 32 consecutive nodes first compute, lanes striding over
// whole particle ranges, every product their loops will add -- a * V/3 for the three lower
// faces, (1 - a) * V/3 for the upper ones -- into shared memory, and the divergent loops then
// only add.  The lower-cell (and own-cell)
// cells of consecutive nodes are consecutive cells, so each of the four roles is one
// contiguous particle range per warp.  A warp whose range exceeds DEP_CAP particles computes
// the products in its loops.  Every sum takes the same values in the same order either way.
constexpr int DEP_WARPS = 8;
constexpr int DEP_CAP = 256;

__global__ void __launch_bounds__(DEP_WARPS * 32) k_deposit_staged(SwarmBuf b, GridDims g,
                                                                    const unsigned int *__restrict__ cs, double third,
                                                                    double *__restrict__ count,
                                                                    double *__restrict__ avg, double *__restrict__ fi,
                                                                    double *__restrict__ fj, double *__restrict__ fk) {
  __shared__ double stage[DEP_WARPS][3][DEP_CAP];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long q = (blockIdx.x * (long long)DEP_WARPS + wid) * 32 + lane;
  if (q - lane >= g.Nn) return;   // the whole warp is past the last node
  const bool node = q < g.Nn;
  const int IM = g.IM, JM = g.JM, KM = g.KM;
  int i = 0, j = 0, k = 0;
  if (node) node_ijk(g, (unsigned int)q, i, j, k);
  const long long c = ((long long)k * JM + j) * IM + i;
  const bool face_i = node && j < JM && k < KM, face_j = node && i < IM && k < KM, face_k = node && i < IM && j < JM;
  const bool is_cell = node && i < IM && j < JM && k < KM;
  // the cell of each role: lower i, lower j, lower k, own (0xffffffff: none)
  const unsigned int NONE = 0xffffffffu;
  unsigned int rc[4];
  rc[0] = (face_i && i > 0) ? (unsigned int)(c - 1) : NONE;
  rc[1] = (face_j && j > 0) ? (unsigned int)(c - IM) : NONE;
  rc[2] = (face_k && k > 0) ? (unsigned int)(c - (long long)IM * JM) : NONE;
  rc[3] = is_cell ? (unsigned int)c : NONE;
  // each role's particle range for the warp: [p0, p1)
  unsigned int p0[4], p1[4];
  bool staged = true;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const unsigned int lo = __reduce_min_sync(0xffffffffu, rc[r]);
    const unsigned int hi = __reduce_max_sync(0xffffffffu, rc[r] == NONE ? 0u : rc[r]);
    p0[r] = 0u;
    p1[r] = 0u;
    if (lo != NONE) {
      p0[r] = __ldg(cs + lo);
      p1[r] = __ldg(cs + hi + 1);
      staged = staged && p1[r] - p0[r] <= (unsigned int)DEP_CAP;
    }
  }
  double acc[3] = {0.0, 0.0, 0.0};
  const double *wgt[3] = {b.a1, b.a2, b.a3};
  if (staged) {
#pragma unroll
    for (int f = 0; f < 3; ++f)
      for (unsigned int s = p0[f] + lane; s < p1[f]; s += 32) stage[wid][f][s - p0[f]] = mul(__ldg(wgt[f] + s), third);
    __syncwarp();
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (rc[f] == NONE) continue;
      const unsigned int l0 = __ldg(cs + rc[f]), l1 = __ldg(cs + rc[f] + 1);
      for (unsigned int s = l0; s < l1; ++s) acc[f] = add(acc[f], stage[wid][f][s - p0[f]]);
    }
    __syncwarp();
  } else {
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      if (rc[f] == NONE) continue;
      const unsigned int l0 = __ldg(cs + rc[f]), l1 = __ldg(cs + rc[f] + 1);
      for (unsigned int s = l0; s < l1; ++s) acc[f] = add(acc[f], mul(__ldg(wgt[f] + s), third));
    }
  }
  // AccumulateParticleField + CalculateParticleCountPerCell + NormalizeGridVectorByCount, and
  // the upper parts of the three faces
  unsigned int s0 = 0u, s1 = 0u;
  if (is_cell) { s0 = __ldg(cs + c); s1 = __ldg(cs + c + 1); }
  double sum = 0.0;
  for (unsigned int s = s0; s < s1; ++s) {
    const double P = __ldg(b.P + s);
    sum = (s == s0) ? fdfx::add0(P) : add(sum, P);
  }
  if (staged) {
    for (unsigned int s = p0[3] + lane; s < p1[3]; s += 32) {
#pragma unroll
      for (int f = 0; f < 3; ++f) stage[wid][f][s - p0[3]] = mul(sub(1.0, __ldg(wgt[f] + s)), third);
    }
    __syncwarp();
    for (unsigned int s = s0; s < s1; ++s) {
#pragma unroll
      for (int f = 0; f < 3; ++f) acc[f] = add(acc[f], stage[wid][f][s - p0[3]]);
    }
  } else {
    for (unsigned int s = s0; s < s1; ++s) {
#pragma unroll
      for (int f = 0; f < 3; ++f) acc[f] = add(acc[f], mul(sub(1.0, __ldg(wgt[f] + s)), third));
    }
  }
  if (!node) return;
  {
    const unsigned int ncell = s1 - s0;   // count += 1.0 per particle is exact in FP64
    count[q] = fdfx::u32_to_double(ncell);
    avg[q] = ncell > 0 ? fdfx::div_count(sum, ncell) : 0.0;
  }
  if (face_i) fi[((long long)k * JM + j) * (IM + 1) + i] = acc[0];   // i-face (i,j,k), i in [0, IM]
  if (face_j) fj[((long long)k * (JM + 1) + j) * IM + i] = acc[1];   // j-face (i,j,k), j in [0, JM]
  if (face_k) fk[c] = acc[2];                                        // k-face (i,j,k), k in [0, KM]
}


// The volume and momentum deposit -- the sums above, bit for bit -- staged like
// k_deposit_staged, one face role at a time: for a lower role, V/3 a and its products with the
// three velocity components; for an upper role, V/3 (1 - a) and its three products.  Each
// role's values for the warp's particle range go to shared memory (four arrays), and the
// per-node loops only add them, each accumulator in the same order.
constexpr int DEPM_WARPS = 4;

__global__ void __launch_bounds__(DEPM_WARPS * 32) k_deposit_mom_staged(SwarmBuf b, GridDims g,
                                                                         const unsigned int *__restrict__ cs,
                                                                         double third, double *__restrict__ count,
                                                                         double *__restrict__ avg,
                                                                         double *__restrict__ fi,
                                                                         double *__restrict__ fj,
                                                                         double *__restrict__ fk,
                                                                         double *__restrict__ mi,
                                                                         double *__restrict__ mj,
                                                                         double *__restrict__ mk) {
  __shared__ double stage[DEPM_WARPS][4][DEP_CAP];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long q = (blockIdx.x * (long long)DEPM_WARPS + wid) * 32 + lane;
  if (q - lane >= g.Nn) return;   // the whole warp is past the last node
  const bool node = q < g.Nn;
  const int IM = g.IM, JM = g.JM, KM = g.KM;
  int i = 0, j = 0, k = 0;
  if (node) node_ijk(g, (unsigned int)q, i, j, k);
  const long long c = ((long long)k * JM + j) * IM + i;
  const bool face_i = node && j < JM && k < KM, face_j = node && i < IM && k < KM, face_k = node && i < IM && j < JM;
  const bool is_cell = node && i < IM && j < JM && k < KM;
  const unsigned int NONE = 0xffffffffu;
  unsigned int rc[4];
  rc[0] = (face_i && i > 0) ? (unsigned int)(c - 1) : NONE;
  rc[1] = (face_j && j > 0) ? (unsigned int)(c - IM) : NONE;
  rc[2] = (face_k && k > 0) ? (unsigned int)(c - (long long)IM * JM) : NONE;
  rc[3] = is_cell ? (unsigned int)c : NONE;
  unsigned int p0[4], p1[4];
  bool staged = true;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const unsigned int lo = __reduce_min_sync(0xffffffffu, rc[r]);
    const unsigned int hi = __reduce_max_sync(0xffffffffu, rc[r] == NONE ? 0u : rc[r]);
    p0[r] = 0u;
    p1[r] = 0u;
    if (lo != NONE) {
      p0[r] = __ldg(cs + lo);
      p1[r] = __ldg(cs + hi + 1);
      staged = staged && p1[r] - p0[r] <= (unsigned int)DEP_CAP;
    }
  }
  const double *wgt[3] = {b.a1, b.a2, b.a3};
  double acc[3] = {0.0, 0.0, 0.0}, mm[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  double (*st)[DEP_CAP] = stage[wid];
  // one role: the values of particle s are (x, x u, x v, x w) with x = V/3 a (lower) or
  // V/3 (1 - a) (upper) of face f; the node's segment is [l0, l1), the warp's [r0, r1)
  auto role = [&](int f, bool upper, unsigned int r0, unsigned int r1, unsigned int l0, unsigned int l1) {
    if (staged) {
      for (unsigned int s = r0 + lane; s < r1; s += 32) {
        const double a = __ldg(wgt[f] + s);
        const double x = mul(upper ? sub(1.0, a) : a, third);
        st[0][s - r0] = x;
        st[1][s - r0] = mul(x, __ldg(b.u + s));
        st[2][s - r0] = mul(x, __ldg(b.v + s));
        st[3][s - r0] = mul(x, __ldg(b.w + s));
      }
      __syncwarp();
      for (unsigned int s = l0; s < l1; ++s) {
        acc[f] = add(acc[f], st[0][s - r0]);
        mm[f][0] = add(mm[f][0], st[1][s - r0]);
        mm[f][1] = add(mm[f][1], st[2][s - r0]);
        mm[f][2] = add(mm[f][2], st[3][s - r0]);
      }
      __syncwarp();
    } else {
      for (unsigned int s = l0; s < l1; ++s) {
        const double a = __ldg(wgt[f] + s);
        const double x = mul(upper ? sub(1.0, a) : a, third);
        acc[f] = add(acc[f], x);
        mm[f][0] = add(mm[f][0], mul(x, __ldg(b.u + s)));
        mm[f][1] = add(mm[f][1], mul(x, __ldg(b.v + s)));
        mm[f][2] = add(mm[f][2], mul(x, __ldg(b.w + s)));
      }
    }
  };
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    unsigned int l0 = 0u, l1 = 0u;
    if (rc[f] != NONE) { l0 = __ldg(cs + rc[f]); l1 = __ldg(cs + rc[f] + 1); }
    role(f, false, p0[f], p1[f], l0, l1);
  }
  unsigned int s0 = 0u, s1 = 0u;
  if (is_cell) { s0 = __ldg(cs + c); s1 = __ldg(cs + c + 1); }
  double sum = 0.0;
  for (unsigned int s = s0; s < s1; ++s) {
    const double P = __ldg(b.P + s);
    sum = (s == s0) ? fdfx::add0(P) : add(sum, P);
  }
#pragma unroll
  for (int f = 0; f < 3; ++f) role(f, true, p0[3], p1[3], s0, s1);
  if (!node) return;
  {
    const unsigned int ncell = s1 - s0;
    count[q] = fdfx::u32_to_double(ncell);
    avg[q] = ncell > 0 ? fdfx::div_count(sum, ncell) : 0.0;
  }
  const long long nfi = (IM + 1LL) * JM * KM, nfj = IM * (JM + 1LL) * KM, nfk = (long long)IM * JM * (KM + 1LL);
  auto store = [&](int f, double *vol, double *mom, long long nf, long long fidx) {
    vol[fidx] = acc[f];
    mom[fidx] = mm[f][0]; mom[nf + fidx] = mm[f][1]; mom[2 * nf + fidx] = mm[f][2];
  };
  if (face_i) store(0, fi, mi, nfi, ((long long)k * JM + j) * (IM + 1) + i);
  if (face_j) store(1, fj, mj, nfj, ((long long)k * (JM + 1) + j) * IM + i);
  if (face_k) store(2, fk, mk, nfk, c);
}

// Slot t of dst takes slot a + t of src for t < b - a, and slot c + (t - (b - a)) after that: the
// held particles of a k-slab ([a, b) in the cell-sorted order) followed by those without a cell
// ([c, n)); every field of both forms moves.
__global__ void k_move_kept(SwarmBuf src, SwarmBuf dst, int a, int b, int c, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = (b - a) + (n - c);
  if (t >= m) return;
  const int p = t < b - a ? a + t : c + (t - (b - a));
  dst.x[t] = src.x[p]; dst.y[t] = src.y[p]; dst.z[t] = src.z[p];
  dst.u[t] = src.u[p]; dst.v[t] = src.v[p]; dst.w[t] = src.w[p];
  dst.a1[t] = src.a1[p]; dst.a2[t] = src.a2[p]; dst.a3[t] = src.a3[p];
  dst.P[t] = src.P[p];
  dst.uf[t] = src.uf[p]; dst.vf[t] = src.vf[p]; dst.wf[t] = src.wf[p];
  dst.a1f[t] = src.a1f[p]; dst.a2f[t] = src.a2f[p]; dst.a3f[t] = src.a3f[p];
  dst.Pf[t] = src.Pf[p];
  dst.pid[t] = src.pid[p];
  dst.cell[t] = src.cell[p];
  dst.status[t] = src.status[p];
}

// The k-faces of layer k (between cells k - 1 and k) summed again from seed values: seed[j][i]
// stands for the lower cell's part of the sum (0.0 + its particles' a V/3 in (cell, PID) order,
// made where the lower cell's particles are held), and the held particles of cell (i, j, k) add
// their (1 - a) V/3 (and its products with the velocity) after it, in sorted order -- the
// single-rank sum, operation for operation.  Momentum seeds are [j][i][3].
__global__ void k_deposit_k_layer(SwarmBuf b, GridDims g, const unsigned int *__restrict__ cs, int k, double third,
                                  const double *__restrict__ seed, const double *__restrict__ seed_mom,
                                  double *__restrict__ fk, double *__restrict__ mk) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;   // (j, i) of the layer
  const long long L = (long long)g.IM * g.JM;
  if (q >= L) return;
  const long long f = (long long)k * L + q;
  double acc = seed[q];
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;
  if (mk) { m0 = seed_mom[3 * q]; m1 = seed_mom[3 * q + 1]; m2 = seed_mom[3 * q + 2]; }
  if (k < g.KM) {
    const unsigned int s0 = __ldg(cs + f), s1 = __ldg(cs + f + 1);
    for (unsigned int s = s0; s < s1; ++s) {
      const double x = mul(sub(1.0, __ldg(b.a3 + s)), third);
      acc = add(acc, x);
      if (mk) {
        m0 = add(m0, mul(x, __ldg(b.u + s)));
        m1 = add(m1, mul(x, __ldg(b.v + s)));
        m2 = add(m2, mul(x, __ldg(b.w + s)));
      }
    }
  }
  fk[f] = acc;
  if (mk) {
    const long long nfk = L * (g.KM + 1LL);
    mk[f] = m0; mk[nfk + f] = m1; mk[2 * nfk + f] = m2;
  }
}

__global__ void k_from_aos(const double *__restrict__ pos, const double *__restrict__ vel,
                           const double *__restrict__ wgt, const double *__restrict__ P,
                           const long long *__restrict__ cell3, const long long *__restrict__ pid,
                           const long long *__restrict__ status, int n, GridDims g, SwarmBuf b) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  b.x[p] = pos[3 * p]; b.y[p] = pos[3 * p + 1]; b.z[p] = pos[3 * p + 2];
  b.u[p] = vel[3 * p]; b.v[p] = vel[3 * p + 1]; b.w[p] = vel[3 * p + 2];
  b.a1[p] = wgt[3 * p]; b.a2[p] = wgt[3 * p + 1]; b.a3[p] = wgt[3 * p + 2];
  b.P[p] = P[p];
  b.pid[p] = pid[p];
  long long i = cell3[3 * p], j = cell3[3 * p + 1], k = cell3[3 * p + 2];
  int c = -1;
  if (i >= 0 && i < g.IM && j >= 0 && j < g.JM && k >= 0 && k < g.KM) c = (int)((k * g.JM + j) * g.IM + i);
  b.cell[p] = c;
  long long st = status[p];
  b.status[p] = (unsigned char)((st >= 0 && st <= ST_UNINITIALIZED) ? st : ST_UNINITIALIZED);
}

__global__ void k_to_aos(SwarmBuf b, int n, GridDims g, double *__restrict__ pos, double *__restrict__ vel,
                         double *__restrict__ wgt, double *__restrict__ P, long long *__restrict__ cell3,
                         long long *__restrict__ pid, long long *__restrict__ status) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  pos[3 * p] = b.x[p]; pos[3 * p + 1] = b.y[p]; pos[3 * p + 2] = b.z[p];
  vel[3 * p] = b.u[p]; vel[3 * p + 1] = b.v[p]; vel[3 * p + 2] = b.w[p];
  wgt[3 * p] = b.a1[p]; wgt[3 * p + 1] = b.a2[p]; wgt[3 * p + 2] = b.a3[p];
  P[p] = b.P[p];
  pid[p] = b.pid[p];
  int c = b.cell[p];
  if (c >= 0) {
    int i, j, k;
    cell_ijk(g, (unsigned int)c, i, j, k);
    cell3[3 * p] = i; cell3[3 * p + 1] = j; cell3[3 * p + 2] = k;
  } else {
    cell3[3 * p] = -1; cell3[3 * p + 1] = -1; cell3[3 * p + 2] = -1;
  }
  status[p] = b.status[p];
}

// ResetAllParticleStatuses (ParticleMotion.c:2149-2176): ACTIVE_AND_LOCATED -> NEEDS_LOCATION.
__global__ void k_reset_status(unsigned char *__restrict__ status, const DevCounters *cnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < cnt->n_sorted && status[s] == ST_ACTIVE_AND_LOCATED) status[s] = ST_NEEDS_LOCATION;
}

// UpdateAllParticlePositions (ParticleMotion.c:38-95): x += v dt per component, as the fused
// step does it.
__global__ void k_advect(SwarmBuf b, double dt, DevCounters *cnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) atomicAdd(&cnt->psteps_total, (unsigned long long)cnt->n_sorted);   // particles advanced
  if (s >= cnt->n_sorted) return;
  b.x[s] = add(b.x[s], mul(b.u[s], dt));
  b.y[s] = add(b.y[s], mul(b.v[s], dt));
  b.z[s] = add(b.z[s], mul(b.w[s], dt));
}

}  // namespace

void launch_reset_status(const SwarmBuf &b, int n_cap, const DevCounters *cnt, cudaStream_t s) {
  k_reset_status<<<(n_cap + 255) / 256 > 0 ? (n_cap + 255) / 256 : 1, 256, 0, s>>>(b.status, cnt);
}

void launch_advect(const SwarmBuf &b, int n_cap, double dt, DevCounters *cnt, cudaStream_t s) {
  k_advect<<<(n_cap + 255) / 256 > 0 ? (n_cap + 255) / 256 : 1, 256, 0, s>>>(b, dt, cnt);
}

void launch_gather_interp(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g, const double *corner,
                          const unsigned int *perm, const unsigned int *cell_start, DevCounters *cnt,
                          cudaStream_t s, int mode) {
  int th = 256;
  int blocks = (n_cap + th - 1) / th;
  if (blocks == 0) blocks = 1;
  k_gather_interp<<<blocks, th, 0, s>>>(src, dst, g, corner, perm, cell_start, cnt, mode);
}

void launch_deposit(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, double volume, double *count,
                    double *avg, double *fi, double *fj, double *fk, double *mi, double *mj, double *mk,
                    cudaStream_t s) {
  const double third = volume / 3.0;
  if (mi)
    k_deposit_mom_staged<<<(unsigned)((g.Nn + DEPM_WARPS * 32 - 1) / (DEPM_WARPS * 32)), DEPM_WARPS * 32, 0, s>>>(
        b, g, cell_start, third, count, avg, fi, fj, fk, mi, mj, mk);
  else
    k_deposit_staged<<<(unsigned)((g.Nn + DEP_WARPS * 32 - 1) / (DEP_WARPS * 32)), DEP_WARPS * 32, 0, s>>>(
        b, g, cell_start, third, count, avg, fi, fj, fk);
}

void launch_move_kept(const SwarmBuf &src, const SwarmBuf &dst, int a, int b, int c, int n, cudaStream_t s) {
  const int m = (b - a) + (n - c);
  if (m <= 0) return;
  k_move_kept<<<(m + 255) / 256, 256, 0, s>>>(src, dst, a, b, c, n);
}

void launch_deposit_k_layer(const SwarmBuf &b, GridDims g, const unsigned int *cell_start, int k, double volume,
                            const double *seed, const double *seed_mom, double *fk, double *mk, cudaStream_t s) {
  const long long L = (long long)g.IM * g.JM;
  k_deposit_k_layer<<<(unsigned)((L + 255) / 256), 256, 0, s>>>(b, g, cell_start, k, volume / 3.0, seed, seed_mom, fk,
                                                                 mk);
}

void launch_swarm_from_aos(const double *pos, const double *vel, const double *wgt, const double *P,
                           const long long *cell3, const long long *pid, const long long *status, int n, GridDims g,
                           const SwarmBuf &b, cudaStream_t s) {
  if (n <= 0) return;
  k_from_aos<<<(n + 255) / 256, 256, 0, s>>>(pos, vel, wgt, P, cell3, pid, status, n, g, b);
}

void launch_swarm_to_aos(const SwarmBuf &b, int n, GridDims g, double *pos, double *vel, double *wgt, double *P,
                         long long *cell3, long long *pid, long long *status, cudaStream_t s) {
  if (n <= 0) return;
  k_to_aos<<<(n + 255) / 256, 256, 0, s>>>(b, n, g, pos, vel, wgt, P, cell3, pid, status);
}
