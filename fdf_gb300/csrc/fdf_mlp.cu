// fdf_mlp.cu -- training of the learned start-cell locator: a 3-128-128-128-3 SiLU MLP
// that maps a particle's physical position to a predicted (i, j, k) cell, trained on
// location pairs produced by the walking search itself.  The walk still decides the cell: the
// prediction is only a starting cell (the learned walk in fdf_fp32.cu); inference runs on
// tcgen05 (fdf_mlp_tc.cu).
//
// Every training GEMM is mma.sync m16n8k16 with bfloat16 operands and FP32 accumulation: a
// generic warp-tile GEMM (16x8 output tile per warp, operands read with arbitrary strides, so
// the same kernel serves X W^T, G W and G^T H), plus elementwise kernels for bias + SiLU, the
// loss, SiLU', bias sums and Adam (FP32 master weights).  Each output is computed by one warp
// in a fixed k order, and the sums run in fixed order, so training is deterministic.  The
// training matrices are small (batch x 128 x 128); the hot path is inference.
//
// Fragment layouts of mma.m16n8k16 (g = lane/4, c = lane%4):
//   A (16x16, row): a0 = A[g][2c..2c+1], a1 = A[g+8][2c..2c+1], a2 = A[g][2c+8..9], a3 = A[g+8][2c+8..9]
//   B (16x8, col):  b0 = B[2c..2c+1][g],  b1 = B[2c+8..9][g]
//   C (16x8, f32):  c0 = C[g][2c], c1 = C[g][2c+1], c2 = C[g+8][2c], c3 = C[g+8][2c+1]
#include "fdf_internal.cuh"
#include "fdf_mlp.cuh"
#include <cuda_bf16.h>
#include <cmath>

namespace {

__device__ __forceinline__ void mma_bf16(float &d0, float &d1, float &d2, float &d3, unsigned a0, unsigned a1,
                                         unsigned a2, unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned *>(&v);
}

__device__ __forceinline__ float bf(const __nv_bfloat16 *p, long long i) { return __bfloat162float(p[i]); }

// SiLU and its derivative in FP32 (training).
__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// ---------------------------------------------------------------- training GEMM
// C(m, n) = sum_k A(m, k) B(k, n), A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn],
// C(m, n) at C[m*scm + n*scn]; one warp per 16x8 tile and K slice of kc (a multiple of 16),
// zero padding outside (M, N, K).  With more than one slice the warps write partial tiles
// [split][M][N] that k_splitk_reduce adds in slice order, so the result does not depend on
// scheduling.
__global__ void k_gemm(const __nv_bfloat16 *__restrict__ A, long long sam, long long sak,
                       const __nv_bfloat16 *__restrict__ B, long long sbk, long long sbn, float *__restrict__ C,
                       long long scm, long long scn, int M, int N, int K, int kc, int splits,
                       float *__restrict__ partials) {
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int tiles_n = (N + 7) / 8, tiles_m = (M + 15) / 16;
  const long long tiles = (long long)tiles_m * tiles_n;
  const int split = (int)(warp / tiles);
  if (split >= splits) return;
  const int t = (int)(warp % tiles);
  const int tm = t / tiles_n, tn = t % tiles_n;
  const int g = lane >> 2, c = lane & 3;
  const int m0 = tm * 16, n0 = tn * 8;
  const int kb = split * kc, ke = min(K, kb + kc);
  float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
  auto Av = [&](int m, int k) -> float { return (m < M && k < ke) ? bf(A, m * sam + k * sak) : 0.f; };
  auto Bv = [&](int k, int n) -> float { return (k < ke && n < N) ? bf(B, k * sbk + n * sbn) : 0.f; };
  for (int k0 = kb; k0 < ke; k0 += 16) {
    const unsigned a0 = pack_bf16(Av(m0 + g, k0 + 2 * c), Av(m0 + g, k0 + 2 * c + 1));
    const unsigned a1 = pack_bf16(Av(m0 + g + 8, k0 + 2 * c), Av(m0 + g + 8, k0 + 2 * c + 1));
    const unsigned a2 = pack_bf16(Av(m0 + g, k0 + 2 * c + 8), Av(m0 + g, k0 + 2 * c + 9));
    const unsigned a3 = pack_bf16(Av(m0 + g + 8, k0 + 2 * c + 8), Av(m0 + g + 8, k0 + 2 * c + 9));
    const unsigned b0 = pack_bf16(Bv(k0 + 2 * c, n0 + g), Bv(k0 + 2 * c + 1, n0 + g));
    const unsigned b1 = pack_bf16(Bv(k0 + 2 * c + 8, n0 + g), Bv(k0 + 2 * c + 9, n0 + g));
    mma_bf16(d0, d1, d2, d3, a0, a1, a2, a3, b0, b1);
  }
  const int r0 = m0 + g, r1 = m0 + g + 8, q0 = n0 + 2 * c, q1 = q0 + 1;
  if (splits == 1) {
    if (r0 < M && q0 < N) C[r0 * scm + q0 * scn] = d0;
    if (r0 < M && q1 < N) C[r0 * scm + q1 * scn] = d1;
    if (r1 < M && q0 < N) C[r1 * scm + q0 * scn] = d2;
    if (r1 < M && q1 < N) C[r1 * scm + q1 * scn] = d3;
  } else {
    float *P = partials + (long long)split * M * N;
    if (r0 < M && q0 < N) P[(long long)r0 * N + q0] = d0;
    if (r0 < M && q1 < N) P[(long long)r0 * N + q1] = d1;
    if (r1 < M && q0 < N) P[(long long)r1 * N + q0] = d2;
    if (r1 < M && q1 < N) P[(long long)r1 * N + q1] = d3;
  }
}

__global__ void k_splitk_reduce(const float *__restrict__ partials, int splits, int M, int N, float *__restrict__ C,
                                long long scm, long long scn) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)M * N) return;
  const long long r = q / N, col = q % N;
  float s = 0.f;
  for (int p = 0; p < splits; ++p) s += partials[(long long)p * M * N + q];
  C[r * scm + col * scn] = s;
}

// ---------------------------------------------------------------- training elementwise
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Minibatch `step`: sample b is mix64(seed, step, b) mod n (with replacement).
__global__ void k_gather_batch(const float *__restrict__ xs, const float *__restrict__ ts, long long n,
                               unsigned long long seed, long long step, int B, __nv_bfloat16 *__restrict__ X,
                               float *__restrict__ T) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const unsigned long long h =
      mix64(mix64(seed * 0xD1B54A32D192ED03ULL + (unsigned long long)step) + (unsigned long long)b * 0x9E3779B97F4A7C15ULL);
  const long long s = (long long)(h % (unsigned long long)n);
  for (int d = 0; d < 3; ++d) {
    X[b * 3 + d] = __float2bfloat16_rn(xs[3 * s + d]);
    T[b * 3 + d] = ts[3 * s + d];
  }
}

__global__ void k_bias_silu(const float *__restrict__ Cin, const float *__restrict__ bias, int B, int N,
                            float *__restrict__ Z, __nv_bfloat16 *__restrict__ H) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)B * N) return;
  const float z = Cin[q] + bias[q % N];
  Z[q] = z;
  H[q] = __float2bfloat16_rn(silu(z));
}

// y = C4 + b4; G = dloss/dy (FP32 and bfloat16); per-block partial sums of the loss
// (squared errors in cells / (3 B), so the partials add up to the batch mean)
__global__ void k_out_loss(const float *__restrict__ C4, const float *__restrict__ b4, const float *__restrict__ T,
                           int B, float sx, float sy, float sz, float *__restrict__ Y, float *__restrict__ G,
                           __nv_bfloat16 *__restrict__ Gb, float *__restrict__ loss_part) {
  __shared__ float red[256];
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (b < B) {
    const float sc[3] = {sx, sy, sz};
    for (int d = 0; d < 3; ++d) {
      const float y = C4[b * 3 + d] + b4[d];
      Y[b * 3 + d] = y;
      const float e = (y - T[b * 3 + d]) * sc[d];
      l += e * e;
      const float gy = 2.0f * e * sc[d] / (3.0f * (float)B);
      G[b * 3 + d] = gy;
      Gb[b * 3 + d] = __float2bfloat16_rn(gy);
    }
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0] / (3.0f * (float)B);
}

__global__ void k_silu_bwd(const float *__restrict__ dH, const float *__restrict__ Z, long long total,
                           float *__restrict__ G, __nv_bfloat16 *__restrict__ Gb) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= total) return;
  const float gv = dH[q] * silu_grad(Z[q]);
  G[q] = gv;
  Gb[q] = __float2bfloat16_rn(gv);
}

// db[n] = sum_b G[b][n]: one warp per column, lanes stride over b, then a fixed-order
// butterfly, so the sum does not depend on scheduling.
__global__ void k_colsum(const float *__restrict__ G, int B, int N, float *__restrict__ db) {
  const int n = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (n >= N) return;
  float s = 0.f;
  for (int b = lane; b < B; b += 32) s += G[(long long)b * N + n];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) db[n] = s;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = g[q];
  const float mq = 0.9f * m[q] + 0.1f * gq;
  const float vq = 0.999f * v[q] + 0.001f * gq * gq;
  m[q] = mq;
  v[q] = vq;
  w[q] = w[q] - lr * (mq / c1) / (sqrtf(vq / c2) + 1e-8f);
}

__global__ void k_to_bf16(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = __float2bfloat16_rn(in[q]);
}

__global__ void k_sum_partials(const float *__restrict__ part, int n, float *__restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  float s = 0.f;
  for (int q = 0; q < n; ++q) s += part[q];
  *out = s;
}

__global__ void k_flag_located(const int *__restrict__ cell, const unsigned char *__restrict__ status, long long n,
                               unsigned int *__restrict__ flag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) flag[q] = (status[q] == ST_ACTIVE_AND_LOCATED && cell[q] >= 0) ? 1u : 0u;
}

__global__ void k_make_samples(const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const int *__restrict__ cell,
                               const unsigned int *__restrict__ slot, const unsigned int *__restrict__ keep,
                               long long n, MlpNorm norm, GridDims g, float *__restrict__ xs,
                               float *__restrict__ ts) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n || !keep[q]) return;
  const long long o = slot[q];
  const double p[3] = {x[q], y[q], z[q]};
  for (int d = 0; d < 3; ++d) xs[3 * o + d] = ((float)p[d] - norm.centre[d]) * norm.inv_half[d];
  int i, j, k;
  cell_ijk(g, (unsigned int)cell[q], i, j, k);
  const int idx[3] = {i, j, k}, N[3] = {g.IM, g.JM, g.KM};
  for (int d = 0; d < 3; ++d) ts[3 * o + d] = 2.0f * ((float)idx[d] + 0.5f) / (float)N[d] - 1.0f;
}

// ---------------------------------------------------------------- inference
// Biases of the four layers in one vector (b1 | b2 | b3 | b4, padded to MLP_BIAS_WORDS).
__global__ void k_pack_bias(const float *__restrict__ params, float *__restrict__ bias) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= MLP_BIAS_WORDS) return;
  float v = 0.f;   // hidden layers: b/2 (the epilogue works on z/2); output layer: b
  if (q < 128) v = 0.5f * params[MLP_OFF_B1 + q];
  else if (q < 256) v = 0.5f * params[MLP_OFF_B2 + q - 128];
  else if (q < 384) v = 0.5f * params[MLP_OFF_B3 + q - 256];
  else if (q < 387) v = params[MLP_OFF_B4 + q - 384];
  bias[q] = v;
}

inline unsigned blocks_for(long long n, int th) { return (unsigned)(n > 0 ? (n + th - 1) / th : 1); }

}  // namespace

// ---------------------------------------------------------------- host side
void mlp_gemm(const __nv_bfloat16 *A, long long sam, long long sak, const __nv_bfloat16 *B, long long sbk,
              long long sbn, float *C, long long scm, long long scn, int M, int N, int K, int splits,
              float *partials, cudaStream_t s) {
  if (splits < 1 || partials == nullptr) splits = 1;
  int kc = (K + splits - 1) / splits;
  kc = (kc + 15) / 16 * 16;
  splits = (K + kc - 1) / kc;
  if (splits < 1) splits = 1;
  const long long warps = (long long)((M + 15) / 16) * ((N + 7) / 8) * splits;
  k_gemm<<<blocks_for(warps * 32, 256), 256, 0, s>>>(A, sam, sak, B, sbk, sbn, C, scm, scn, M, N, K, kc, splits,
                                                     partials);
  if (splits > 1)
    k_splitk_reduce<<<blocks_for((long long)M * N, 256), 256, 0, s>>>(partials, splits, M, N, C, scm, scn);
}

void mlp_gather_batch(const float *xs, const float *ts, long long n_samples, unsigned long long seed, long long step,
                      int B, __nv_bfloat16 *X, float *T, cudaStream_t s) {
  k_gather_batch<<<blocks_for(B, 256), 256, 0, s>>>(xs, ts, n_samples, seed, step, B, X, T);
}
void mlp_bias_silu(const float *C, const float *b, int B, int N, float *Z, __nv_bfloat16 *H, cudaStream_t s) {
  k_bias_silu<<<blocks_for((long long)B * N, 256), 256, 0, s>>>(C, b, B, N, Z, H);
}
void mlp_out_loss(const float *C4, const float *b4, const float *T, int B, const float sc[3], float *Y, float *G,
                  __nv_bfloat16 *Gb, float *loss_part, cudaStream_t s) {
  k_out_loss<<<blocks_for(B, 256), 256, 0, s>>>(C4, b4, T, B, sc[0], sc[1], sc[2], Y, G, Gb, loss_part);
}
void mlp_silu_bwd(const float *dH, const float *Z, long long total, float *G, __nv_bfloat16 *Gb, cudaStream_t s) {
  k_silu_bwd<<<blocks_for(total, 256), 256, 0, s>>>(dH, Z, total, G, Gb);
}
void mlp_colsum(const float *G, int B, int N, float *db, cudaStream_t s) {
  k_colsum<<<blocks_for((long long)N * 32, 256), 256, 0, s>>>(G, B, N, db);
}
void mlp_adam(float *w, const float *g, float *m, float *v, int n, float lr, float c1, float c2, cudaStream_t s) {
  k_adam<<<blocks_for(n, 256), 256, 0, s>>>(w, g, m, v, n, lr, c1, c2);
}
void mlp_to_bf16(const float *in, __nv_bfloat16 *out, int n, cudaStream_t s) {
  k_to_bf16<<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
}
void mlp_sum_partials(const float *part, int n, float *out, cudaStream_t s) {
  k_sum_partials<<<1, 32, 0, s>>>(part, n, out);
}
void mlp_pack_bias(const float *params, float *bias, cudaStream_t s) {
  k_pack_bias<<<blocks_for(MLP_BIAS_WORDS, 256), 256, 0, s>>>(params, bias);
}
void mlp_flag_located(const int *cell, const unsigned char *status, long long n, unsigned int *flag, cudaStream_t s) {
  k_flag_located<<<blocks_for(n, 256), 256, 0, s>>>(cell, status, n, flag);
}
void mlp_make_samples(const double *x, const double *y, const double *z, const int *cell, const unsigned int *slot,
                      const unsigned int *keep, long long n, MlpNorm norm, GridDims g, float *xs, float *ts,
                      cudaStream_t s) {
  k_make_samples<<<blocks_for(n, 256), 256, 0, s>>>(x, y, z, cell, slot, keep, n, norm, g, xs, ts);
}

namespace {
unsigned long long mix64_host(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double uniform01_host(unsigned long long seed, unsigned long long stream, unsigned long long idx) {
  const unsigned long long base =
      mix64_host(seed * 0xD1B54A32D192ED03ULL + stream * 0xA24BAED4963EE407ULL + 0x632BE59BD9B4E019ULL);
  const unsigned long long z = mix64_host(base + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
}  // namespace

void mlp_init_params_host(unsigned long long seed, float *params) {
  const int sizes[5] = {3, MLP_H, MLP_H, MLP_H, 3};
  const int offw[4] = {MLP_OFF_W1, MLP_OFF_W2, MLP_OFF_W3, MLP_OFF_W4};
  const int offb[4] = {MLP_OFF_B1, MLP_OFF_B2, MLP_OFF_B3, MLP_OFF_B4};
  for (int L = 0; L < 4; ++L) {
    const int fin = sizes[L], fout = sizes[L + 1];
    const double scale = std::sqrt((double)fin);
    for (int q = 0; q < fin * fout; ++q)
      params[offw[L] + q] = (float)((2.0 * uniform01_host(seed, 100 + L, (unsigned long long)q) - 1.0) / scale);
    for (int q = 0; q < fout; ++q) params[offb[L] + q] = 0.0f;
  }
}
