// fdf_mlp.cu -- training of the learned start-cell locator: a 3-128-128-128-3 SiLU MLP
// that maps a particle's physical position to a predicted (i, j, k) cell, trained on
// location pairs produced by the walking search itself.  The walk still decides the cell: the
// prediction is only a starting cell (the learned walk in fdf_fp32.cu); inference runs on
// tcgen05 (fdf_mlp_tc.cu).
//
// Every training GEMM runs on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// bfloat16 operands, FP32 accumulator in tensor memory): one generic GEMM kernel whose CTAs
// stage 128-row tiles of both operands -- read with arbitrary strides, so the same kernel
// serves X W^T, G W and G^T H -- into shared memory in the K-major core-matrix layout
// (fdf_tc.cuh), 64 K columns at a time, and let one thread issue the chunk's four MMAs; plus
// elementwise kernels for bias + SiLU, the loss, SiLU', bias sums and Adam (FP32 master
// weights).  Each output is accumulated by one CTA in a fixed K order, split-K partials and
// the other sums are added in fixed order, so training is deterministic.  The training
// matrices are small (batch x 128 x 128); the hot path is inference.
//
// Input layer.  Each normalised coordinate enters as the bfloat16 pair hi = bf16(x),
// lo = bf16(x - hi) (K = 6: hi x, y, z, lo x, y, z) against W1 repeated in both column groups,
// as in inference; the W1 gradient is the sum of the two groups' gradients.
#include "fdf_internal.cuh"
#include "fdf_mlp.cuh"
#include "fdf_tc.cuh"
#include <cuda_bf16.h>
#include <cmath>

namespace {

// SiLU and its derivative in FP32 (training).
__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// ---------------------------------------------------------------- training GEMM
// C(m, n) = sum_k A(m, k) B(k, n), A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn],
// C(m, n) at C[m*scm + n*scn].  One CTA per 128 x NT output tile (NT = 16 for N <= 16, else
// 128) and K slice [kb, kb + kc): its 128 threads stage A's rows and B's columns for 64 K at a
// time (zeros outside M, N, K) as the A [128][64] and B [NT][64] operands, thread 0 issues
// four M = 128 MMAs of K = 16 into the CTA's 128 TMEM columns, and everyone waits on the
// mbarrier before the next chunk overwrites the operands.  The four warps then read their
// 32 accumulator lanes (rows).  With more than one slice the CTAs write partial tiles
// [split][M][N] that k_splitk_reduce adds in slice order, so the result does not depend on
// scheduling.  A wait that runs out sets ERRBIT_TC_TIMEOUT in *err; the CTA then frees its
// tensor memory and returns without writing.
constexpr int GT_KC = 64;
constexpr int GT_THREADS = 128;
constexpr int GT_SM_A = 0;               // [128][64] bfloat16, 16 KB
constexpr int GT_SM_B = 16384;           // [128][64] bfloat16, 16 KB
constexpr int GT_SM_BAR = 32768;         // mbarrier (8 B), TMEM base (4 B), time-out flag (4 B)
// dynamic shared memory asked per CTA: at most three CTAs share an SM, 3 x 128 of its 512 TMEM
// columns, so no allocation ever waits
constexpr int GT_SM_LAUNCH = 72 * 1024;
constexpr unsigned long long GT_WAIT_LIMIT = 1ull << 22;

__device__ __forceinline__ unsigned short bf_bits(const __nv_bfloat16 *p, long long i) {
  return reinterpret_cast<const unsigned short *>(p)[i];
}

__global__ void __launch_bounds__(GT_THREADS)
    k_gemm_tc(const __nv_bfloat16 *__restrict__ A, long long sam, long long sak, const __nv_bfloat16 *__restrict__ B,
              long long sbk, long long sbn, float *__restrict__ C, long long scm, long long scn, int M, int N, int K,
              int kc, int splits, float *__restrict__ partials, unsigned int *__restrict__ err,
              unsigned long long wait_limit) {
  using namespace fdftc;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nt = N <= 16 ? 16 : 128;
  const int tiles_n = (N + nt - 1) / nt, tiles_m = (M + 127) / 128;
  const int t = (int)(blockIdx.x % (unsigned)(tiles_m * tiles_n)), split = (int)(blockIdx.x / (unsigned)(tiles_m * tiles_n));
  const int m0 = (t / tiles_n) * 128, n0 = (t % tiles_n) * nt;
  const int kb = split * kc, ke = min(K, kb + kc);
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(smem + GT_SM_BAR + 8);
  volatile unsigned *tflag = reinterpret_cast<volatile unsigned *>(smem + GT_SM_BAR + 12);
  const unsigned bar_addr = smem_u32(smem + GT_SM_BAR);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_addr) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *tflag = 0u;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const unsigned tmem = *tmem_slot;
  const unsigned a_addr = smem_u32(smem + GT_SM_A), b_addr = smem_u32(smem + GT_SM_B);
  const unsigned idesc = make_idesc(128, nt, true);
  unsigned phase = 0;
  bool ok = true;
#pragma unroll 1
  for (int k0 = kb; k0 < ke && ok; k0 += GT_KC) {
    // 8 consecutive K columns of one row per item, stored as one 16-B line of a core matrix
#pragma unroll 1
    for (int q = tid; q < 128 * 8; q += GT_THREADS) {
      const int r = q >> 3, kg = (q & 7) * 8, m = m0 + r;
      unsigned short v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = k0 + kg + e;
        v[e] = (m < M && k < ke) ? bf_bits(A, m * sam + k * sak) : (unsigned short)0;
      }
      *reinterpret_cast<uint4 *>(smem + GT_SM_A + op_off(r, kg, 16 * GT_KC)) =
          make_uint4(v[0] | ((unsigned)v[1] << 16), v[2] | ((unsigned)v[3] << 16), v[4] | ((unsigned)v[5] << 16),
                     v[6] | ((unsigned)v[7] << 16));
    }
#pragma unroll 1
    for (int q = tid; q < nt * 8; q += GT_THREADS) {
      const int r = q >> 3, kg = (q & 7) * 8, n = n0 + r;
      unsigned short v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int k = k0 + kg + e;
        v[e] = (n < N && k < ke) ? bf_bits(B, k * sbk + n * sbn) : (unsigned short)0;
      }
      *reinterpret_cast<uint4 *>(smem + GT_SM_B + op_off(r, kg, 16 * GT_KC)) =
          make_uint4(v[0] | ((unsigned)v[1] << 16), v[2] | ((unsigned)v[3] << 16), v[4] | ((unsigned)v[5] << 16),
                     v[6] | ((unsigned)v[7] << 16));
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
#pragma unroll
      for (int s = 0; s < GT_KC / 16; ++s)
        mma_f16(tmem, make_desc(a_addr + 256 * s, 128, 16 * GT_KC), make_desc(b_addr + 256 * s, 128, 16 * GT_KC),
                idesc, (k0 > kb || s > 0) ? 1u : 0u);
      mma_commit(bar_addr);
    }
    // the chunk's MMAs read the staged operands: they finish before the next chunk is staged
    bool done = false;
    for (unsigned long long it = 0; it < wait_limit && !done; ++it) done = mbar_try_wait(bar_addr, phase);
    phase ^= 1u;
    if (!done) *tflag = 1u;
    __syncthreads();
    ok = *tflag == 0u;
    fence_after_sync();
  }
  if (ok) {
    const int m = m0 + 32 * warp + lane;   // warp w reads TMEM lanes 32w .. 32w + 31
#pragma unroll 1
    for (int c = 0; c < nt; c += 16) {
      float v[16];
      tmem_ld16(tmem + ((unsigned)(32 * warp) << 16) + (unsigned)c, v);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int n = n0 + c + q;
        if (m < M && n < N) {
          if (splits == 1) C[m * scm + n * scn] = v[q];
          else partials[((long long)split * M + m) * N + n] = v[q];
        }
      }
    }
  } else if (tid == 0) {
    atomicOr(err, (unsigned)ERRBIT_TC_TIMEOUT);
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(128) : "memory");
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

// The bfloat16 pair (hi, lo) of a normalised coordinate: X row [hi x, y, z, lo x, y, z].
__device__ __forceinline__ void split_row(const float *x, __nv_bfloat16 *X) {
  for (int d = 0; d < 3; ++d) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x[d]);
    X[d] = h;
    X[3 + d] = __float2bfloat16_rn(x[d] - __bfloat162float(h));
  }
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
  split_row(xs + 3 * s, X + 6 * b);
  for (int d = 0; d < 3; ++d) T[b * 3 + d] = ts[3 * s + d];
}

__global__ void k_split_inputs(const float *__restrict__ xs, int B, __nv_bfloat16 *__restrict__ X) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) split_row(xs + 3 * b, X + 6 * b);
}

// W1 [128][3] (bfloat16) repeated as W1x [128][6] = [W1 | W1]; and the W1 gradient as the sum of
// the two column groups' gradients dW1x [128][6].
__global__ void k_split_w1(const __nv_bfloat16 *__restrict__ w1, __nv_bfloat16 *__restrict__ w1x) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < MLP_H * 6) w1x[q] = w1[(q / 6) * 3 + (q % 6) % 3];
}
__global__ void k_fold_w1(const float *__restrict__ dw1x, float *__restrict__ dw1) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < MLP_H * 3) dw1[q] = dw1x[(q / 3) * 6 + q % 3] + dw1x[(q / 3) * 6 + 3 + q % 3];
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
              float *partials, unsigned int *err, cudaStream_t s) {
  static int attr_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (attr_device != dev) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GT_SM_LAUNCH);
    attr_device = dev;
  }
  if (splits < 1 || partials == nullptr) splits = 1;
  int kc = (K + splits - 1) / splits;
  kc = (kc + GT_KC - 1) / GT_KC * GT_KC;
  splits = (K + kc - 1) / kc;
  if (splits < 1) splits = 1;
  const int nt = N <= 16 ? 16 : 128;
  const long long ctas = (long long)((M + 127) / 128) * ((N + nt - 1) / nt) * splits;
  k_gemm_tc<<<(unsigned)ctas, GT_THREADS, GT_SM_LAUNCH, s>>>(A, sam, sak, B, sbk, sbn, C, scm, scn, M, N, K, kc,
                                                             splits, partials, err, GT_WAIT_LIMIT);
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
void mlp_split_inputs(const float *xs, int B, __nv_bfloat16 *X, cudaStream_t s) {
  k_split_inputs<<<blocks_for(B, 256), 256, 0, s>>>(xs, B, X);
}
void mlp_split_w1(const __nv_bfloat16 *w1, __nv_bfloat16 *w1x, cudaStream_t s) {
  k_split_w1<<<blocks_for(MLP_H * 6, 256), 256, 0, s>>>(w1, w1x);
}
void mlp_fold_w1(const float *dw1x, float *dw1, cudaStream_t s) {
  k_fold_w1<<<blocks_for(MLP_H * 3, 256), 256, 0, s>>>(dw1x, dw1);
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
