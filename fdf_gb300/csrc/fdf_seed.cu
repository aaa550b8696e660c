// fdf_seed.cu -- on-device volumetric particle seeding for large synthetic workloads.
//
// Restates, on the GPU, the harness generator of fdf_gb300/workloads.py
// (volumetric_particles): the reference's volumetric initialisation
// (ParticleSwarm.c:229-312) -- a random cell, random logical coordinates in [0,1)
// clamped to 1 - 1e-7 -- mapped to physical space by the trilinear blend of
// Metric.c:48-62, with the same counter-based splitmix64 streams and the same FP64
// operation order (no FMA), so the particles are bit-identical to the host's.
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// uniform01(seed, stream)[idx] of workloads.py
__device__ __forceinline__ double uniform01(unsigned long long seed, unsigned long long stream,
                                            unsigned long long idx) {
  const unsigned long long base =
      mix64(seed * 0xD1B54A32D192ED03ULL + stream * 0xA24BAED4963EE407ULL + 0x632BE59BD9B4E019ULL);
  const unsigned long long z = mix64(base + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_seed(const double *__restrict__ coor, GridDims g, long long n, unsigned long long seed,
                       long long pid_base, int hint, int form32, double P0, SwarmBuf b) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const unsigned long long idx = (unsigned long long)p;
  const double ri = uniform01(seed, 0, idx), rj = uniform01(seed, 1, idx), rk = uniform01(seed, 2, idx);
  long long ci = (long long)fdfx::mul(ri, (double)g.IM), cj = (long long)fdfx::mul(rj, (double)g.JM),
            ck = (long long)fdfx::mul(rk, (double)g.KM);
  ci = ci < 0 ? 0 : (ci > g.IM - 1 ? g.IM - 1 : ci);
  cj = cj < 0 ? 0 : (cj > g.JM - 1 ? g.JM - 1 : cj);
  ck = ck < 0 ? 0 : (ck > g.KM - 1 ? g.KM - 1 : ck);
  const double lim = 1.0 - 1.0e-7;
  double xi = uniform01(seed, 3, idx), eta = uniform01(seed, 4, idx), zta = uniform01(seed, 5, idx);
  xi = fdfx::pmax(fdfx::pmin(xi, lim), 0.0);     // np.maximum(np.minimum(u, lim), 0.0) on [0,1) values
  eta = fdfx::pmax(fdfx::pmin(eta, lim), 0.0);
  zta = fdfx::pmax(fdfx::pmin(zta, lim), 0.0);
  double x = 0.0, y = 0.0, z = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const double a = (c & 1) ? xi : fdfx::sub(1.0, xi);
    const double bb = (c & 2) ? eta : fdfx::sub(1.0, eta);
    const double cc = (c & 4) ? zta : fdfx::sub(1.0, zta);
    const double N = fdfx::mul(fdfx::mul(a, bb), cc);
    const long long ii = ci + ((c & 1) ? 1 : 0), jj = cj + ((c & 2) ? 1 : 0), kk = ck + ((c & 4) ? 1 : 0);
    const double *V = coor + 3 * ((kk * (g.JM + 1) + jj) * (long long)(g.IM + 1) + ii);
    x = fdfx::add(x, fdfx::mul(N, V[0]));
    y = fdfx::add(y, fdfx::mul(N, V[1]));
    z = fdfx::add(z, fdfx::mul(N, V[2]));
  }
  if (form32) {
    const double v[3] = {x, y, z};
    double *dst[3] = {b.x, b.y, b.z};
    for (int q = 0; q < 3; ++q) {
      const float h = __double2float_rn(v[q]);
      const float l = __double2float_rn(__dsub_rn(v[q], (double)h));
      *reinterpret_cast<float2 *>(dst[q] + p) = make_float2(h, l);
    }
    b.uf[p] = 0.f; b.vf[p] = 0.f; b.wf[p] = 0.f;
    b.a1f[p] = 0.f; b.a2f[p] = 0.f; b.a3f[p] = 0.f;
    b.Pf[p] = (float)P0;
  } else {
    b.x[p] = x; b.y[p] = y; b.z[p] = z;
    b.u[p] = 0.0; b.v[p] = 0.0; b.w[p] = 0.0;
    b.a1[p] = 0.0; b.a2[p] = 0.0; b.a3[p] = 0.0;
    b.P[p] = P0;
  }
  b.pid[p] = pid_base + p;
  b.cell[p] = hint ? (int)((ck * g.JM + cj) * g.IM + ci) : -1;
  b.status[p] = ST_UNINITIALIZED;
}

}  // namespace

void launch_seed(const double *coor, GridDims g, long long n, unsigned long long seed, long long pid_base, int hint,
                 int form32, double P0, const SwarmBuf &b, cudaStream_t s) {
  if (n <= 0) return;
  k_seed<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(coor, g, n, seed, pid_base, hint, form32, P0, b);
}
