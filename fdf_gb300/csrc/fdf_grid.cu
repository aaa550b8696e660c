// fdf_grid.cu -- grid-side kernels: per-cell face-plane table, center->corner
// averaging of ucat, bounding box.
//
// All FP64 arithmetic on the parity path uses the _rn intrinsics, which the
// compiler never contracts into an FMA, so every value is rounded exactly as the
// reference (compiled without FMA) rounds it.
#include "fdf_internal.cuh"
#include <cfloat>

namespace {

struct V3 { double x, y, z; };

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ V3 node(const double *coor, GridDims g, long long i, long long j, long long k) {
  const double *q = coor + 3 * ((k * (g.JM + 1) + j) * (long long)(g.IM + 1) + i);
  return V3{q[0], q[1], q[2]};
}

// One face of ComputeSignedDistanceToPlane (walkingsearch.c:102-227) with every
// particle-independent quantity evaluated: face centroid and oriented unit normal.
__device__ __forceinline__ bool face_plane(V3 v1, V3 v2, V3 v3, V3 v4, V3 cc, double *row) {
  double e1x = sub(v2.x, v1.x), e1y = sub(v2.y, v1.y), e1z = sub(v2.z, v1.z);
  double e2x = sub(v4.x, v1.x), e2y = sub(v4.y, v1.y), e2z = sub(v4.z, v1.z);
  double nxi = sub(mul(e1y, e2z), mul(e1z, e2y));
  double nyi = sub(mul(e1z, e2x), mul(e1x, e2z));
  double nzi = sub(mul(e1x, e2y), mul(e1y, e2x));
  double mag = __dsqrt_rn(add(add(mul(nxi, nxi), mul(nyi, nyi)), mul(nzi, nzi)));
  bool degenerate = mag < 1.0e-12;
  double fcx = mul(0.25, add(add(add(v1.x, v2.x), v3.x), v4.x));
  double fcy = mul(0.25, add(add(add(v1.y, v2.y), v3.y), v4.y));
  double fcz = mul(0.25, add(add(add(v1.z, v2.z), v3.z), v4.z));
  double tx = sub(cc.x, fcx), ty = sub(cc.y, fcy), tz = sub(cc.z, fcz);
  double dot = add(add(mul(nxi, tx), mul(nyi, ty)), mul(nzi, tz));
  double nx = nxi, ny = nyi, nz = nzi;
  if (dot > 1.0e-9) { nx = -nxi; ny = -nyi; nz = -nzi; }
  row[0] = fcx; row[1] = fcy; row[2] = fcz;
  row[3] = __ddiv_rn(nx, mag); row[4] = __ddiv_rn(ny, mag); row[5] = __ddiv_rn(nz, mag);
  return degenerate;
}

__global__ void k_build_planes(const double *__restrict__ coor, GridDims g, double *__restrict__ planes,
                               unsigned int *err) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= g.Nc) return;
  long long i = c % g.IM, t = c / g.IM, j = t % g.JM, k = t / g.JM;
  // walkingsearch.c:521-549 vertex numbering
  V3 v[8];
  v[0] = node(coor, g, i, j, k);         v[1] = node(coor, g, i + 1, j, k);
  v[2] = node(coor, g, i + 1, j + 1, k); v[3] = node(coor, g, i, j + 1, k);
  v[4] = node(coor, g, i, j + 1, k + 1); v[5] = node(coor, g, i + 1, j + 1, k + 1);
  v[6] = node(coor, g, i + 1, j, k + 1); v[7] = node(coor, g, i, j, k + 1);
  // GetCellCharacteristicSize, walkingsearch.c:25-59
  const int e[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                        {6, 7}, {7, 4}, {0, 7}, {1, 6}, {2, 5}, {3, 4}};
  double total = 0.0;
#pragma unroll
  for (int q = 0; q < 12; ++q) {
    V3 A = v[e[q][0]], B = v[e[q][1]];
    double dx = sub(B.x, A.x), dy = sub(B.y, A.y), dz = sub(B.z, A.z);
    total = add(total, __dsqrt_rn(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz))));
  }
  double h = __ddiv_rn(total, 12.0);
  double thr = mul(FDF_DISTANCE_THRESHOLD, h);
  // cell centroid, walkingsearch.c:286-296
  V3 cc{0.0, 0.0, 0.0};
#pragma unroll
  for (int q = 0; q < 8; ++q) { cc.x = add(cc.x, v[q].x); cc.y = add(cc.y, v[q].y); cc.z = add(cc.z, v[q].z); }
  cc.x = __ddiv_rn(cc.x, 8.0); cc.y = __ddiv_rn(cc.y, 8.0); cc.z = __ddiv_rn(cc.z, 8.0);
  double *row = planes + c * FDF_ROW;
  bool degen = false;
  // face vertex lists, walkingsearch.c:303-378
  degen |= face_plane(v[0], v[3], v[2], v[1], cc, row + 6 * F_BACK);
  degen |= face_plane(v[4], v[7], v[6], v[5], cc, row + 6 * F_FRONT);
  degen |= face_plane(v[0], v[1], v[6], v[7], cc, row + 6 * F_BOTTOM);
  degen |= face_plane(v[3], v[4], v[5], v[2], cc, row + 6 * F_TOP);
  degen |= face_plane(v[0], v[7], v[4], v[3], cc, row + 6 * F_LEFT);
  degen |= face_plane(v[1], v[2], v[5], v[6], cc, row + 6 * F_RIGHT);
  row[36] = thr;
  row[37] = degen ? 1.0 : 0.0;
  (void)err;
}

// InterpolateFieldFromCenterToCorner_Vector_Petsc, interpolation.c:598-679.
// Each node averages its valid adjacent cells in (dk, dj, di) order; the count is
// 1, 2, 4 or 8, so sum/count equals sum*(1/count) exactly.
__global__ void k_center_to_corner(const double *__restrict__ ucat, GridDims g, double *__restrict__ corner) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= g.Nn) return;
  const long long mx = g.IM + 1, my = g.JM + 1;
  long long i = q % mx, t = q / mx, j = t % my, k = t / my;
  const double *ux = ucat, *uy = ucat + g.Nc, *uz = ucat + 2 * g.Nc;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  int count = 0;
#pragma unroll
  for (int dk = -1; dk <= 0; ++dk) {
    long long ck = k + dk;
    if (ck < 0 || ck >= g.KM) continue;
#pragma unroll
    for (int dj = -1; dj <= 0; ++dj) {
      long long cj = j + dj;
      if (cj < 0 || cj >= g.JM) continue;
#pragma unroll
      for (int di = -1; di <= 0; ++di) {
        long long ci = i + di;
        if (ci < 0 || ci >= g.IM) continue;
        long long c = (ck * g.JM + cj) * g.IM + ci;
        sx = add(sx, __ldg(ux + c)); sy = add(sy, __ldg(uy + c)); sz = add(sz, __ldg(uz + c));
        ++count;
      }
    }
  }
  double ox = 0.0, oy = 0.0, oz = 0.0;
  if (count > 0) {
    double dc = (double)count;
    ox = __ddiv_rn(sx, dc); oy = __ddiv_rn(sy, dc); oz = __ddiv_rn(sz, dc);
  }
  corner[q] = ox; corner[g.Nn + q] = oy; corner[2 * g.Nn + q] = oz;
}

__device__ __forceinline__ double atomic_min_d(double *addr, double val) {
  unsigned long long *a = (unsigned long long *)addr;
  unsigned long long old = *a, assumed;
  do {
    assumed = old;
    if (__longlong_as_double(assumed) <= val) break;
    old = atomicCAS(a, assumed, __double_as_longlong(val));
  } while (assumed != old);
  return __longlong_as_double(old);
}
__device__ __forceinline__ double atomic_max_d(double *addr, double val) {
  unsigned long long *a = (unsigned long long *)addr;
  unsigned long long old = *a, assumed;
  do {
    assumed = old;
    if (__longlong_as_double(assumed) >= val) break;
    old = atomicCAS(a, assumed, __double_as_longlong(val));
  } while (assumed != old);
  return __longlong_as_double(old);
}

// ComputeLocalBoundingBox, grid.c:762-883 (min/max over nodes; the widening by
// 1e-6 is applied by the host). min/max are order-independent, so atomics are exact.
__global__ void k_bbox(const double *__restrict__ coor, long long nn, double *bbox6) {
  double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mxv[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nn;
       q += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double v = coor[3 * q + c];
      if (v < mn[c]) mn[c] = v;
      if (v > mxv[c]) mxv[c] = v;
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    for (int o = 16; o > 0; o >>= 1) {
      double a = __shfl_down_sync(0xffffffffu, mn[c], o);
      double b = __shfl_down_sync(0xffffffffu, mxv[c], o);
      if (a < mn[c]) mn[c] = a;
      if (b > mxv[c]) mxv[c] = b;
    }
    if ((threadIdx.x & 31) == 0) { atomic_min_d(&bbox6[c], mn[c]); atomic_max_d(&bbox6[3 + c], mxv[c]); }
  }
}

}  // namespace

void launch_build_planes(const double *coor, GridDims g, double *planes, unsigned int *err, cudaStream_t s) {
  int th = 128;
  long long blocks = (g.Nc + th - 1) / th;
  k_build_planes<<<(unsigned)blocks, th, 0, s>>>(coor, g, planes, err);
}

void launch_center_to_corner(const double *ucat, GridDims g, double *corner, cudaStream_t s) {
  int th = 256;
  long long blocks = (g.Nn + th - 1) / th;
  k_center_to_corner<<<(unsigned)blocks, th, 0, s>>>(ucat, g, corner);
}

void launch_bbox(const double *coor, long long nn, double *bbox6, cudaStream_t s) {
  k_bbox<<<152 * 4, 256, 0, s>>>(coor, nn, bbox6);
}
