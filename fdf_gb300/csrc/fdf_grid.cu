// fdf_grid.cu -- grid-side kernels: per-cell face-plane table and center->corner
// averaging of ucat.
//
// All FP64 arithmetic on the parity path uses the _rn intrinsics, which the
// compiler never contracts into an FMA, so every value is rounded exactly as the
// reference (compiled without FMA) rounds it.
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"
#include "fdf_counters.cuh"
#include <cfloat>

namespace {

struct V3 { double x, y, z; };

using fdfx::add;
using fdfx::sub;
using fdfx::mul;

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
  int i, j, k;
  cell_ijk(g, (unsigned int)c, i, j, k);
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
// Each node averages its valid adjacent cells in (dk, dj, di) order.  The count is
// a product of per-direction counts of 1 or 2, i.e. 1, 2, 4 or 8, so sum/count is
// exactly sum*(1/count): both are the correctly rounded value of the same real.
// The running sum starts at 0.0; "0.0 + first" is the first value except that a
// -0.0 becomes +0.0 (add0).  With cell_start non-null, nodes none of whose
// adjacent cells holds a particle are skipped: the corner field is an
// intermediate of the interpolation and only those nodes are ever read.
__global__ void k_center_to_corner(const double *__restrict__ ucat, GridDims g, double *__restrict__ corner,
                                   const unsigned int *__restrict__ cell_start, unsigned long long *nodes_done) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool work = q < g.Nn;
  if (cell_start) {
    // count the nodes this step computes (for the roofline bytes)
    bool need = false;
    if (work) {
      int i0, j0, k0;
      node_ijk(g, (unsigned int)q, i0, j0, k0);
      for (int dk = -1; dk <= 0 && !need; ++dk)
        for (int dj = -1; dj <= 0 && !need; ++dj)
          for (int di = -1; di <= 0 && !need; ++di) {
            int ck = k0 + dk, cj = j0 + dj, ci = i0 + di;
            if (ci < 0 || ci >= g.IM || cj < 0 || cj >= g.JM || ck < 0 || ck >= g.KM) continue;
            long long c = ((long long)ck * g.JM + cj) * g.IM + ci;
            need = __ldg(cell_start + c + 1) > __ldg(cell_start + c);
          }
    }
    if (nodes_done) block_add_u64(need ? 1ull : 0ull, nodes_done);
    if (!need) return;
  }
  if (!work) return;
  int i, j, k;
  node_ijk(g, (unsigned int)q, i, j, k);
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
        double vx = __ldg(ux + c), vy = __ldg(uy + c), vz = __ldg(uz + c);
        if (count == 0) {
          sx = fdfx::add0(vx); sy = fdfx::add0(vy); sz = fdfx::add0(vz);
        } else {
          sx = add(sx, vx); sy = add(sy, vy); sz = add(sz, vz);
        }
        ++count;
      }
    }
  }
  double ox = 0.0, oy = 0.0, oz = 0.0;
  if (count > 0) {
    const int sh = count == 1 ? 0 : count == 2 ? 1 : count == 4 ? 2 : 3;   // sum * 0.5^sh, exact
    ox = fdfx::scale_down(sx, sh); oy = fdfx::scale_down(sy, sh); oz = fdfx::scale_down(sz, sh);
  }
  corner[q] = ox; corner[g.Nn + q] = oy; corner[2 * g.Nn + q] = oz;
}

}  // namespace

void launch_build_planes(const double *coor, GridDims g, double *planes, unsigned int *err, cudaStream_t s) {
  int th = 128;
  long long blocks = (g.Nc + th - 1) / th;
  k_build_planes<<<(unsigned)blocks, th, 0, s>>>(coor, g, planes, err);
}

void launch_center_to_corner(const double *ucat, GridDims g, double *corner, const unsigned int *cell_start,
                             unsigned long long *nodes_done, cudaStream_t s) {
  int th = 256;
  long long blocks = (g.Nn + th - 1) / th;
  k_center_to_corner<<<(unsigned)blocks, th, 0, s>>>(ucat, g, corner, cell_start, nodes_done);
}
