// fdf_eulerian.cu -- the Eulerian input of the particle path on the device: the grid's face
// metrics and inverse Jacobian, the orientation check, and Contra2Cart (contravariant face
// velocity -> cell-centred Cartesian ucat), for callers whose ucat changes every step.
//
//   ComputeFaceMetrics          Metric.c:286-460  Csi, Eta, Zet at every node + extrapolation
//   ComputeCellCenteredJacobianInverse  Metric.c:491-600  Aj = 1/J + extrapolation
//   CheckAndFixGridOrientation  Metric.c:195-260  mixed signs -> error, all negative -> flip
//   Contra2Cart                 setup.c:1294-1420 Cramer's rule per interior cell
//
// Every value is computed with the reference's operations in its order (no FMA contraction:
// the library is built with --fmad=false), so metrics and ucat are bit-identical to it.
//
// Design: the metrics depend only on the grid, and so do the Cramer's-rule determinant and
// the nine 2x2 minors it shares with det0..det2.  They are computed once per grid into a
// per-cell table [11][Nc] (1/det, the minors of det0, det1, det2, then 1/(2 det)); a
// Contra2Cart call reads 80 B of table and the face velocities per cell and does 21 FP64
// operations (3 face sums, 9 products, 6 sums, 3 scalings) instead of ~90 plus a division, and
// converts its FP32 copy on the integer pipe.  The table holds the reference's intermediate
// values exactly, and the halved form is exact in the range it is used, so every bit of ucat is
// the reference's.  The kernel is bound by GB300's FP64 pipe, not HBM.
#include "fdf_context.cuh"
#include "fdf_exact.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int C2C_SLOTS = 11;            // 1/det | A0 A1 A2 | B0 B1 B2 | C0 C1 C2 | 1/(2 det)
constexpr unsigned ERR_JACOBIAN = 1u;    // |J| < 1e-12 at a node (Metric.c:560)
constexpr unsigned ERR_DET = 2u;         // |det| < 1e-18 in a cell (setup.c:1389-1391)
constexpr unsigned ERR_WIDE = 4u;        // a tabled value outside [2^-400, 2^400] (not an error)

// |x| in [2^-400, 2^400], or x == +-0: products of two such values neither overflow nor leave
// the normal range, so halving them (and their sums) is exact.
__device__ __forceinline__ bool mid_range(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) << 1;   // sign dropped
  const unsigned int e = (unsigned int)(b >> 53);
  return b == 0ull || (e - (1023u - 400u)) <= 800u;
}

using fdfx::d2f_rn;   // double -> float on the integer pipe

__device__ __forceinline__ long long nid(const GridDims &g, int i, int j, int k) {
  return ((long long)k * (g.JM + 1) + j) * (g.IM + 1) + i;
}

// Face metrics and the inverse Jacobian of one node.  Outputs start zeroed; a component the
// reference does not compute at this node (its stencil would leave the grid) stays zero.
__global__ void k_metrics(const double *__restrict__ coor, GridDims g, double *__restrict__ csi,
                          double *__restrict__ eta, double *__restrict__ zet, double *__restrict__ aj,
                          unsigned *__restrict__ err) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.Nn) return;
  int i, j, k;
  node_ijk(g, (unsigned)n, i, j, k);
  auto P = [&](int c, int ii, int jj, int kk) { return coor[3 * nid(g, ii, jj, kk) + c]; };
  if (j >= 1 && k >= 1) {   // Csi, Metric.c:325-341
    double de[3], dz[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      de[c] = 0.5 * (P(c, i, j, k) + P(c, i, j, k - 1) - P(c, i, j - 1, k) - P(c, i, j - 1, k - 1));
      dz[c] = 0.5 * (P(c, i, j - 1, k) + P(c, i, j, k) - P(c, i, j - 1, k - 1) - P(c, i, j, k - 1));
    }
    csi[3 * n] = de[1] * dz[2] - de[2] * dz[1];
    csi[3 * n + 1] = de[2] * dz[0] - de[0] * dz[2];
    csi[3 * n + 2] = de[0] * dz[1] - de[1] * dz[0];
  }
  if (k >= 1 && i >= 1) {   // Eta, Metric.c:344-360
    double dx[3], dz[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dx[c] = 0.5 * (P(c, i, j, k) + P(c, i, j, k - 1) - P(c, i - 1, j, k) - P(c, i - 1, j, k - 1));
      dz[c] = 0.5 * (P(c, i, j, k) + P(c, i - 1, j, k) - P(c, i, j, k - 1) - P(c, i - 1, j, k - 1));
    }
    eta[3 * n] = dz[1] * dx[2] - dz[2] * dx[1];
    eta[3 * n + 1] = dz[2] * dx[0] - dz[0] * dx[2];
    eta[3 * n + 2] = dz[0] * dx[1] - dz[1] * dx[0];
  }
  if (j >= 1 && i >= 1) {   // Zet, Metric.c:363-379
    double dx[3], de[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dx[c] = 0.5 * (P(c, i, j, k) + P(c, i, j - 1, k) - P(c, i - 1, j, k) - P(c, i - 1, j - 1, k));
      de[c] = 0.5 * (P(c, i, j, k) + P(c, i - 1, j, k) - P(c, i, j - 1, k) - P(c, i - 1, j - 1, k));
    }
    zet[3 * n] = dx[1] * de[2] - dx[2] * de[1];
    zet[3 * n + 1] = dx[2] * de[0] - dx[0] * de[2];
    zet[3 * n + 2] = dx[0] * de[1] - dx[1] * de[0];
  }
  if (i >= 1 && j >= 1 && k >= 1) {   // Aj, Metric.c:527-562
    double dxi[3], deta[3], dzeta[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dxi[c] = 0.25 * ((P(c, i, j, k) + P(c, i, j - 1, k) + P(c, i, j, k - 1) + P(c, i, j - 1, k - 1)) -
                       (P(c, i - 1, j, k) + P(c, i - 1, j - 1, k) + P(c, i - 1, j, k - 1) + P(c, i - 1, j - 1, k - 1)));
      deta[c] = 0.25 * ((P(c, i, j, k) + P(c, i - 1, j, k) + P(c, i, j, k - 1) + P(c, i - 1, j, k - 1)) -
                        (P(c, i, j - 1, k) + P(c, i - 1, j - 1, k) + P(c, i, j - 1, k - 1) + P(c, i - 1, j - 1, k - 1)));
      dzeta[c] = 0.25 * ((P(c, i, j, k) + P(c, i, j - 1, k) + P(c, i - 1, j, k) + P(c, i - 1, j - 1, k)) -
                         (P(c, i, j, k - 1) + P(c, i, j - 1, k - 1) + P(c, i - 1, j, k - 1) + P(c, i - 1, j - 1, k - 1)));
    }
    const double J = dxi[0] * (deta[1] * dzeta[2] - deta[2] * dzeta[1]) -
                     dxi[1] * (deta[0] * dzeta[2] - deta[2] * dzeta[0]) +
                     dxi[2] * (deta[0] * dzeta[1] - deta[1] * dzeta[0]);
    if (fabs(J) < 1.0e-12) atomicOr(err, ERR_JACOBIAN);
    aj[n] = 1.0 / J;
  }
}

// Boundary extrapolation of one logical direction (Metric.c:383-452 and 570-620): on every
// grid line along `dir`, node 0 takes node 1's value, then the last node the one before it.
// dir 0 copies Eta, Zet (and Aj); dir 1 Csi, Zet, Aj; dir 2 Csi, Eta, Aj.  The three
// directions run as three launches in the reference's order.
__global__ void k_extrapolate(GridDims g, int dir, double *__restrict__ v1, double *__restrict__ v2,
                              double *__restrict__ aj) {
  const int mx = g.IM + 1, my = g.JM + 1, mz = g.KM + 1;
  const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int m = dir == 0 ? mx : dir == 1 ? my : mz;
  const long long lines = dir == 0 ? (long long)my * mz : dir == 1 ? (long long)mx * mz : (long long)mx * my;
  if (line >= lines) return;
  long long base, stride;
  if (dir == 0) {
    const int j = (int)(line % my), k = (int)(line / my);
    base = nid(g, 0, j, k); stride = 1;
  } else if (dir == 1) {
    const int i = (int)(line % mx), k = (int)(line / mx);
    base = nid(g, i, 0, k); stride = mx;
  } else {
    const int i = (int)(line % mx), j = (int)(line / mx);
    base = nid(g, i, j, 0); stride = (long long)mx * my;
  }
  auto copy = [&](long long dst, long long src) {
#pragma unroll
    for (int c = 0; c < 3; ++c) { v1[3 * dst + c] = v1[3 * src + c]; v2[3 * dst + c] = v2[3 * src + c]; }
    aj[dst] = aj[src];
  };
  if (1 < m) copy(base, base + stride);
  if (m - 2 >= 0) copy(base + (long long)(m - 1) * stride, base + (long long)(m - 2) * stride);
}

// Per-block min and max of Aj (VecMin / VecMax, Metric.c:210-211); the host finishes.
__global__ void k_minmax(const double *__restrict__ a, long long n, double *__restrict__ part) {
  __shared__ double slo[256], shi[256];
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  double lo = inf, hi = -inf;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double v = a[q];
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  slo[threadIdx.x] = lo; shi[threadIdx.x] = hi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      slo[threadIdx.x] = fmin(slo[threadIdx.x], slo[threadIdx.x + s]);
      shi[threadIdx.x] = fmax(shi[threadIdx.x], shi[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = slo[0]; part[2 * blockIdx.x + 1] = shi[0]; }
}

// VecScale(-1) of Csi, Eta, Zet ([3][Nn][3] contiguous) and Aj (Metric.c:229-233).
__global__ void k_negate(double *__restrict__ a, long long n) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) a[q] = -a[q];
}

// The grid-only part of Contra2Cart (setup.c:1357-1395) per interior cell: the matrix of
// face-averaged metrics, its determinant (|det| < 1e-18 is the reference's error), 1/det and
// the nine 2x2 minors det0..det2 multiply by, in the reference's operation order.
__global__ void k_c2c_table(const double *__restrict__ csi, const double *__restrict__ eta,
                            const double *__restrict__ zet, GridDims g, double *__restrict__ table,
                            unsigned *__restrict__ err) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.Nc) return;
  int i, j, k;
  cell_ijk(g, (unsigned)c, i, j, k);
  double t[C2C_SLOTS];
#pragma unroll
  for (int s = 0; s < C2C_SLOTS; ++s) t[s] = 0.0;
  if (i >= 1 && j >= 1 && k >= 1) {
    const long long n = nid(g, i, j, k), ni = nid(g, i - 1, j, k), nj = nid(g, i, j - 1, k), nk = nid(g, i, j, k - 1);
    double m[3][3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      m[0][q] = 0.5 * (csi[3 * ni + q] + csi[3 * n + q]);
      m[1][q] = 0.5 * (eta[3 * nj + q] + eta[3 * n + q]);
      m[2][q] = 0.5 * (zet[3 * nk + q] + zet[3 * n + q]);
    }
    const double A0 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    const double A1 = m[0][1] * m[2][2] - m[0][2] * m[2][1];
    const double A2 = m[0][1] * m[1][2] - m[0][2] * m[1][1];
    const double B0 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
    const double B1 = m[0][0] * m[2][2] - m[0][2] * m[2][0];
    const double B2 = m[0][0] * m[1][2] - m[0][2] * m[1][0];
    const double C0 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const double C1 = m[0][0] * m[2][1] - m[0][1] * m[2][0];
    const double C2 = m[0][0] * m[1][1] - m[0][1] * m[1][0];
    // det's three minors are the same expressions as A0, B0 and C0 (setup.c:1383-1385)
    const double det = m[0][0] * A0 - m[0][1] * B0 + m[0][2] * C0;
    if (fabs(det) < 1.0e-18) atomicOr(err, ERR_DET);
    t[0] = 1.0 / det;
    t[1] = A0; t[2] = A1; t[3] = A2;
    t[4] = B0; t[5] = B1; t[6] = B2;
    t[7] = C0; t[8] = C1; t[9] = C2;
    t[10] = 0.5 * t[0];
    bool mid = t[0] != 0.0 && mid_range(t[0]);
#pragma unroll
    for (int q = 1; q < 10; ++q) mid = mid && mid_range(t[q]);
    if (!mid) atomicOr(err, ERR_WIDE);
  }
#pragma unroll
  for (int s = 0; s < C2C_SLOTS; ++s) table[s * g.Nc + c] = t[s];
}

// Contra2Cart (setup.c:1374-1409) of the interior cells: the face-averaged contravariant
// velocity q, det0..det2 from the tabled minors, ucat = det_q / det.  Writes the FP64 ucat
// (SoA [3][Nc]) and its FP32 copy; boundary cells keep their values.
//
// HALF (every tabled value in [2^-400, 2^400]): with s = a + b, the reference's q = s/2 and
// det0 = q0 A0 - q1 A1 + q2 A2 are exactly half of s0 A0 - s1 A1 + s2 A2 whenever the face
// sums s lie in [2^-400, 2^400] too (products and sums stay normal, so halving commutes with
// every rounding), and det0 * (1/det) then rounds the same real number as
// (s0 A0 - s1 A1 + s2 A2) * (1/(2 det)).  Three FP64 multiplications per cell fewer; a cell
// whose face sums fall outside that range takes the reference's literal sequence.
// The reference's literal sequence (setup.c:1374-1409) from the face sums; out of line so that
// the compiler does not if-convert its halvings into the common path.
__device__ __noinline__ void c2c_literal(double s0, double s1, double s2, const double *__restrict__ table,
                                         long long c, long long N, double &u, double &v, double &w) {
  const double q0 = 0.5 * s0, q1 = 0.5 * s1, q2 = 0.5 * s2;
  const double di = table[c];
  u = (q0 * table[N + c] - q1 * table[2 * N + c] + q2 * table[3 * N + c]) * di;
  v = (-q0 * table[4 * N + c] + q1 * table[5 * N + c] - q2 * table[6 * N + c]) * di;
  w = (q0 * table[7 * N + c] - q1 * table[8 * N + c] + q2 * table[9 * N + c]) * di;
}

template <bool HALF>
__global__ void __launch_bounds__(256) k_contra2cart(const double *__restrict__ ucont, const double *__restrict__ table,
                                                     GridDims g, double *__restrict__ ucat, float *__restrict__ ucat32) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.Nc) return;
  int i, j, k;
  cell_ijk(g, (unsigned)c, i, j, k);
  if (i == 0 || j == 0 || k == 0) return;
  const long long n = nid(g, i, j, k);
  const long long sj = g.IM + 1, sk = (long long)(g.IM + 1) * (g.JM + 1);
  const double s0 = ucont[3 * (n - 1)] + ucont[3 * n];
  const double s1 = ucont[3 * (n - sj) + 1] + ucont[3 * n + 1];
  const double s2 = ucont[3 * (n - sk) + 2] + ucont[3 * n + 2];
  const long long N = g.Nc;
  double u, v, w;
  if (HALF && mid_range(s0) && mid_range(s1) && mid_range(s2)) {
    const double hdi = table[10 * N + c];
    u = (s0 * table[N + c] - s1 * table[2 * N + c] + s2 * table[3 * N + c]) * hdi;
    v = (-s0 * table[4 * N + c] + s1 * table[5 * N + c] - s2 * table[6 * N + c]) * hdi;
    w = (s0 * table[7 * N + c] - s1 * table[8 * N + c] + s2 * table[9 * N + c]) * hdi;
  } else {
    c2c_literal(s0, s1, s2, table, c, N, u, v, w);
  }
  ucat[c] = u; ucat[N + c] = v; ucat[2 * N + c] = w;
  ucat32[c] = d2f_rn(u); ucat32[N + c] = d2f_rn(v); ucat32[2 * N + c] = d2f_rn(w);
}

inline unsigned blocks_of(long long n, int th) { return (unsigned)((n + th - 1) / th); }

// Face metrics [3][Nn][3] (Csi | Eta | Zet) and Aj [Nn] of the context's grid on the device,
// orientation checked and fixed like the reference.  The caller frees *metrics and *aj.
int device_metrics(FdfContext *ctx, double **metrics, double **aj, int *flipped) {
  const GridDims &g = ctx->g;
  const long long Nn = g.Nn;
  *metrics = nullptr; *aj = nullptr;
  double *m = nullptr, *a = nullptr, *part = nullptr;
  unsigned *err = nullptr;
  constexpr int MM_BLOCKS = 1024;
  auto cleanup = [&]() { cfree(m); cfree(a); cfree(part); cfree(err); };
  cudaError_t e = cudaMalloc((void **)&m, 72ull * Nn);
  if (e == cudaSuccess) e = cudaMalloc((void **)&a, 8ull * Nn);
  if (e == cudaSuccess) e = cudaMalloc((void **)&part, 16ull * MM_BLOCKS);
  if (e == cudaSuccess) e = cudaMalloc((void **)&err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(m, 0, 72ull * Nn, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(a, 0, 8ull * Nn, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream);
  if (e != cudaSuccess) {
    cleanup();
    return fail(ctx, e == cudaErrorMemoryAllocation ? FDF_ERR_MEM : FDF_ERR_GPU,
                std::string("grid metrics: ") + cudaGetErrorString(e));
  }
  double *csi = m, *eta = m + 3 * Nn, *zet = m + 6 * Nn;
  k_metrics<<<blocks_of(Nn, 256), 256, 0, ctx->stream>>>(ctx->coor, g, csi, eta, zet, a, err);
  const long long mx = g.IM + 1, my = g.JM + 1, mz = g.KM + 1;
  k_extrapolate<<<blocks_of(my * mz, 256), 256, 0, ctx->stream>>>(g, 0, eta, zet, a);
  k_extrapolate<<<blocks_of(mx * mz, 256), 256, 0, ctx->stream>>>(g, 1, csi, zet, a);
  k_extrapolate<<<blocks_of(mx * my, 256), 256, 0, ctx->stream>>>(g, 2, csi, eta, a);
  const int mm_blocks = (int)std::min<long long>(MM_BLOCKS, (Nn + 255) / 256);
  k_minmax<<<mm_blocks, 256, 0, ctx->stream>>>(a, Nn, part);
  ctx->launches += 6;
  unsigned err_h = 0;
  std::vector<double> part_h(2 * (size_t)mm_blocks);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err_h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part_h.data(), part, 16ull * mm_blocks, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cleanup();
    return fail(ctx, FDF_ERR_GPU, std::string("grid metrics: ") + cudaGetErrorString(e));
  }
  if (err_h & ERR_JACOBIAN) {
    cleanup();
    return fail(ctx, FDF_ERR_FLOP_COUNT, "ComputeCellCenteredJacobianInverse: Jacobian is near zero");
  }
  double lo = part_h[0], hi = part_h[1];
  for (int b = 1; b < mm_blocks; ++b) { lo = std::fmin(lo, part_h[2 * b]); hi = std::fmax(hi, part_h[2 * b + 1]); }
  if (lo < 0.0 && hi > 0.0) {
    cleanup();
    return fail(ctx, FDF_ERR_USER, "CheckAndFixGridOrientation: mixed Jacobian signs, the grid is inconsistent");
  }
  *flipped = 0;
  if (hi < 0.0) {   // a left-handed grid: flip every metric vector and Aj
    k_negate<<<blocks_of(9 * Nn, 256), 256, 0, ctx->stream>>>(m, 9 * Nn);
    k_negate<<<blocks_of(Nn, 256), 256, 0, ctx->stream>>>(a, Nn);
    ctx->launches += 2;
    *flipped = 1;
  }
  e = cudaGetLastError();
  cfree(part); cfree(err);
  if (e != cudaSuccess) {
    cleanup();
    return fail(ctx, FDF_ERR_GPU, std::string("grid metrics: ") + cudaGetErrorString(e));
  }
  *metrics = m; *aj = a;
  return FDF_SUCCESS;
}

// The per-cell Contra2Cart table of the current grid, built on first use.
int ensure_c2c_table(FdfContext *ctx) {
  if (ctx->c2c_table) return ctx->c2c_rc == FDF_SUCCESS ? FDF_SUCCESS : fail(ctx, ctx->c2c_rc, ctx->c2c_msg);
  const GridDims &g = ctx->g;
  double *m = nullptr, *a = nullptr;
  int flipped = 0;
  int r = device_metrics(ctx, &m, &a, &flipped);
  if (r) return r;
  unsigned *err = nullptr;
  cudaError_t e = cudaMalloc((void **)&ctx->c2c_table, 8ull * C2C_SLOTS * g.Nc);
  if (e == cudaSuccess) e = cudaMalloc((void **)&err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream);
  if (e == cudaSuccess) {
    k_c2c_table<<<blocks_of(g.Nc, 256), 256, 0, ctx->stream>>>(m, m + 3 * g.Nn, m + 6 * g.Nn, g, ctx->c2c_table, err);
    ctx->launches += 1;
    e = cudaGetLastError();
  }
  unsigned err_h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err_h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cfree(m); cfree(a); cfree(err);
  if (e != cudaSuccess) {
    cfree(ctx->c2c_table);
    return fail(ctx, e == cudaErrorMemoryAllocation ? FDF_ERR_MEM : FDF_ERR_GPU,
                std::string("Contra2Cart table: ") + cudaGetErrorString(e));
  }
  ctx->c2c_flipped = flipped;
  ctx->c2c_half = (err_h & ERR_WIDE) == 0u;
  ctx->c2c_rc = FDF_SUCCESS;
  if (err_h & ERR_DET) {
    ctx->c2c_rc = FDF_ERR_FLOP_COUNT;
    ctx->c2c_msg = "Contra2Cart: transformation matrix determinant is near zero";
    return fail(ctx, ctx->c2c_rc, ctx->c2c_msg);
  }
  return FDF_SUCCESS;
}

}  // namespace

void eulerian_free(FdfContext *ctx) {
  cfree(ctx->c2c_table);
  cfree(ctx->ucont);
  ctx->c2c_rc = FDF_SUCCESS;
  ctx->c2c_msg.clear();
  ctx->c2c_flipped = 0;
  ctx->c2c_half = false;
}

extern "C" {

int fdf_GetGridMetrics(FdfContext *ctx, double *csi, double *eta, double *zet, double *aj, int *flipped) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetGridMetrics: call fdf_SetGrid first");
  CU(cudaSetDevice(ctx->device));
  double *m = nullptr, *a = nullptr;
  int fl = 0;
  int r = device_metrics(ctx, &m, &a, &fl);
  if (r) return r;
  const long long Nn = ctx->g.Nn;
  cudaError_t e = cudaSuccess;
  double *outs[3] = {csi, eta, zet};
  for (int q = 0; q < 3 && e == cudaSuccess; ++q)
    if (outs[q]) e = cudaMemcpyAsync(outs[q], m + 3 * q * Nn, 24ull * Nn, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && aj) e = cudaMemcpyAsync(aj, a, 8ull * Nn, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cfree(m); cfree(a);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_GetGridMetrics: ") + cudaGetErrorString(e));
  if (flipped) *flipped = fl;
  return FDF_SUCCESS;
}

int fdf_SetUcont(FdfContext *ctx, const double *ucont) {
  if (!ctx || !ucont) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_SetUcont: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_SetUcont: call fdf_SetGrid first");
  CU(cudaSetDevice(ctx->device));
  if (!ctx->ucont) CU(cudaMalloc((void **)&ctx->ucont, 24ull * ctx->g.Nn));
  CU(cudaMemcpyAsync(ctx->ucont, ucont, 24ull * ctx->g.Nn, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

}  // extern "C"

namespace {

// The conversion of a face-velocity array in device memory (the context's copy or the caller's).
int contra2cart_from(FdfContext *ctx, const double *ucont) {
  CU(cudaSetDevice(ctx->device));
  int r = ensure_c2c_table(ctx);
  if (r) return r;
  const bool prof = ctx->profiling;
  const size_t e0 = prof ? record_event(ctx, ctx->stream) : 0;
  if (ctx->c2c_half)
    k_contra2cart<true><<<blocks_of(ctx->g.Nc, 256), 256, 0, ctx->stream>>>(ucont, ctx->c2c_table, ctx->g, ctx->ucat,
                                                                          ctx->ucat32);
  else
    k_contra2cart<false><<<blocks_of(ctx->g.Nc, 256), 256, 0, ctx->stream>>>(ucont, ctx->c2c_table, ctx->g,
                                                                           ctx->ucat, ctx->ucat32);
  CHECK_LAUNCH();
  ctx->launches += 1;
  if (prof) {
    const size_t e1 = record_event(ctx, ctx->stream);
    ctx->ev_spans.push_back({FDF_STAGE_CONTRA2CART, {e0, e1}});
  }
  ctx->has_ucat = true;
  return FDF_SUCCESS;
}

}  // namespace

extern "C" {

int fdf_Contra2Cart(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid || !ctx->ucont)   // setup.c:1311-1313
    return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_Contra2Cart: requires the grid and the face velocity (fdf_SetUcont)");
  return contra2cart_from(ctx, ctx->ucont);
}

int fdf_Contra2CartDevice(FdfContext *ctx, const double *ucont_device) {
  if (!ctx || !ucont_device) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_Contra2CartDevice: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_Contra2CartDevice: call fdf_SetGrid first");
  cudaPointerAttributes at{};
  CU(cudaPointerGetAttributes(&at, ucont_device));
  if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != ctx->device)
    return fail(ctx, FDF_ERR_ARG_WRONG, "fdf_Contra2CartDevice: the face velocity is not in this context's device memory");
  return contra2cart_from(ctx, ucont_device);
}

int fdf_GetUcat(FdfContext *ctx, double *ucat, int node_sized) {
  if (!ctx || !ucat) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetUcat: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetUcat: call fdf_SetGrid first");
  const GridDims &g = ctx->g;
  CU(cudaSetDevice(ctx->device));
  std::vector<double> soa(3 * (size_t)g.Nc);
  CU(cudaMemcpyAsync(soa.data(), ctx->ucat, 24ull * g.Nc, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  const long long mx = node_sized ? g.IM + 1 : g.IM, my = node_sized ? g.JM + 1 : g.JM;
  if (node_sized) memset(ucat, 0, 24ull * g.Nn);
  for (long long k = 0; k < g.KM; ++k)
    for (long long j = 0; j < g.JM; ++j)
      for (long long i = 0; i < g.IM; ++i) {
        const long long c = (k * g.JM + j) * g.IM + i;
        double *v = ucat + 3 * ((k * my + j) * mx + i);
        v[0] = soa[c]; v[1] = soa[g.Nc + c]; v[2] = soa[2 * g.Nc + c];
      }
  return FDF_SUCCESS;
}

}  // extern "C"
