// fdf_particles.cu -- grid-to-particle interpolation fused with the sorted
// gather, the deterministic particle-to-grid deposits, and the DMSwarm AoS <->
// device SoA marshalling.
#include "fdf_internal.cuh"

namespace {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
// PETSc's PetscMin / PetscMax macros: a<b ? a : b and a<b ? b : a.
__device__ __forceinline__ double pmin(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double pmax(double a, double b) { return (a < b) ? b : a; }

// Sorted slot s takes the particle from slot vals[s] of the previous order, then
// interpolates ucat to it: ComputeTrilinearWeights (interpolation.c:839-864) and
// TrilinearInterpolation_Vector (:957-1042) from the node-averaged field, with
// the stencil guard of InterpolateEulerFieldToSwarm (:1356-1372).
__global__ void __launch_bounds__(256) k_gather_interp(SwarmBuf src, SwarmBuf dst, GridDims g,
                                                       const double *__restrict__ corner,
                                                       const unsigned int *__restrict__ keys,
                                                       const unsigned int *__restrict__ vals, unsigned int sentinel,
                                                       const DevCounters *cnt) {
  const int n = cnt->n_sorted;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const unsigned int key = keys[s];
  const unsigned int p = vals[s];
  double a1 = src.a1[p], a2 = src.a2[p], a3 = src.a3[p];
  dst.x[s] = src.x[p]; dst.y[s] = src.y[p]; dst.z[s] = src.z[p];
  dst.a1[s] = a1; dst.a2[s] = a2; dst.a3[s] = a3;
  dst.P[s] = src.P[p];
  dst.pid[s] = src.pid[p];
  double ux = 0.0, uy = 0.0, uz = 0.0;
  if (key >= sentinel) {
    dst.cell[s] = -1;
    dst.status[s] = ST_LOST;
  } else {
    dst.cell[s] = (int)key;
    dst.status[s] = ST_ACTIVE_AND_LOCATED;
    const int i = (int)(key % (unsigned)g.IM);
    const unsigned int t = key / (unsigned)g.IM;
    const int j = (int)(t % (unsigned)g.JM), k = (int)(t / (unsigned)g.JM);
    a1 = pmax(0.0, pmin(1.0, a1));
    a2 = pmax(0.0, pmin(1.0, a2));
    a3 = pmax(0.0, pmin(1.0, a3));
    const double oa1 = sub(1.0, a1), oa2 = sub(1.0, a2), oa3 = sub(1.0, a3);
    double w[8];
    w[0] = mul(mul(oa1, oa2), oa3); w[1] = mul(mul(a1, oa2), oa3);
    w[2] = mul(mul(oa1, a2), oa3);  w[3] = mul(mul(a1, a2), oa3);
    w[4] = mul(mul(oa1, oa2), a3);  w[5] = mul(mul(a1, oa2), a3);
    w[6] = mul(mul(oa1, a2), a3);   w[7] = mul(mul(a1, a2), a3);
    const long long mx = g.IM + 1, my = g.JM + 1;
    const long long q0 = ((long long)k * my + j) * mx + i;
    const long long off[8] = {0, 1, mx, mx + 1, mx * my, mx * my + 1, mx * my + mx, mx * my + mx + 1};
    const double *cx = corner, *cy = corner + g.Nn, *cz = corner + 2 * g.Nn;
    double sw = 0.0, ax = 0.0, ay = 0.0, az = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const long long q = q0 + off[c];
      ax = add(ax, mul(w[c], __ldg(cx + q)));
      ay = add(ay, mul(w[c], __ldg(cy + q)));
      az = add(az, mul(w[c], __ldg(cz + q)));
      sw = add(sw, w[c]);
    }
    if (sw > 1.0e-14) {
      ux = __ddiv_rn(ax, sw); uy = __ddiv_rn(ay, sw); uz = __ddiv_rn(az, sw);
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
__global__ void __launch_bounds__(256) k_deposit(SwarmBuf b, GridDims g, const int *__restrict__ cs,
                                                 double third, double *__restrict__ count,
                                                 double *__restrict__ avg, double *__restrict__ fi,
                                                 double *__restrict__ fj, double *__restrict__ fk) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nn) return;
  const int IM = g.IM, JM = g.JM, KM = g.KM;
  const long long mx = IM + 1, my = JM + 1;
  const int i = (int)(q % mx);
  const long long t = q / mx;
  const int j = (int)(t % my), k = (int)(t / my);
  const bool is_cell = i < IM && j < JM && k < KM;
  const long long c = ((long long)k * JM + j) * IM + i;
  int s0 = 0, s1 = 0;
  if (is_cell) { s0 = __ldg(cs + c); s1 = __ldg(cs + c + 1); }
  // AccumulateParticleField + CalculateParticleCountPerCell + NormalizeGridVectorByCount
  {
    double sum = 0.0, cntv = 0.0;
    for (int s = s0; s < s1; ++s) { sum = add(sum, __ldg(b.P + s)); cntv = add(cntv, 1.0); }
    count[q] = cntv;
    avg[q] = (cntv > 0.5) ? __ddiv_rn(sum, cntv) : 0.0;
  }
  if (j < JM && k < KM) {   // i-face (i,j,k), i in [0, IM]
    double acc = 0.0;
    if (i > 0) {
      long long cl = c - 1;
      int l0 = __ldg(cs + cl), l1 = __ldg(cs + cl + 1);
      for (int s = l0; s < l1; ++s) acc = add(acc, mul(__ldg(b.a1 + s), third));
    }
    if (i < IM)
      for (int s = s0; s < s1; ++s) acc = add(acc, mul(sub(1.0, __ldg(b.a1 + s)), third));
    fi[((long long)k * JM + j) * (IM + 1) + i] = acc;
  }
  if (i < IM && k < KM) {   // j-face (i,j,k), j in [0, JM]
    double acc = 0.0;
    if (j > 0) {
      long long cl = ((long long)k * JM + (j - 1)) * IM + i;
      int l0 = __ldg(cs + cl), l1 = __ldg(cs + cl + 1);
      for (int s = l0; s < l1; ++s) acc = add(acc, mul(__ldg(b.a2 + s), third));
    }
    if (j < JM)
      for (int s = s0; s < s1; ++s) acc = add(acc, mul(sub(1.0, __ldg(b.a2 + s)), third));
    fj[((long long)k * (JM + 1) + j) * IM + i] = acc;
  }
  if (i < IM && j < JM) {   // k-face (i,j,k), k in [0, KM]
    double acc = 0.0;
    if (k > 0) {
      long long cl = ((long long)(k - 1) * JM + j) * IM + i;
      int l0 = __ldg(cs + cl), l1 = __ldg(cs + cl + 1);
      for (int s = l0; s < l1; ++s) acc = add(acc, mul(__ldg(b.a3 + s), third));
    }
    if (k < KM)
      for (int s = s0; s < s1; ++s) acc = add(acc, mul(sub(1.0, __ldg(b.a3 + s)), third));
    fk[c] = acc;
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
    long long i = c % g.IM, t = c / g.IM;
    cell3[3 * p] = i; cell3[3 * p + 1] = t % g.JM; cell3[3 * p + 2] = t / g.JM;
  } else {
    cell3[3 * p] = -1; cell3[3 * p + 1] = -1; cell3[3 * p + 2] = -1;
  }
  status[p] = b.status[p];
}

}  // namespace

void launch_gather_interp(const SwarmBuf &src, const SwarmBuf &dst, int n_cap, GridDims g, const double *corner,
                              const unsigned int *keys, const unsigned int *vals, unsigned int sentinel,
                              const DevCounters *cnt, cudaStream_t s) {
  int th = 256;
  int blocks = (n_cap + th - 1) / th;
  if (blocks == 0) blocks = 1;
  k_gather_interp<<<blocks, th, 0, s>>>(src, dst, g, corner, keys, vals, sentinel, cnt);
}

void launch_deposit(const SwarmBuf &b, GridDims g, const int *cell_start, double volume, double *count, double *avg,
                    double *fi, double *fj, double *fk, cudaStream_t s) {
  int th = 256;
  long long blocks = (g.Nn + th - 1) / th;
  double third = volume / 3.0;
  k_deposit<<<(unsigned)blocks, th, 0, s>>>(b, g, cell_start, third, count, avg, fi, fj, fk);
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
