// fdf_mlp.cu -- training of the learned start-cell locator: a 3-128-128-128-3 SiLU MLP
// that maps a particle's physical position to a predicted (i, j, k) cell, trained on
// location pairs produced by the walking search itself.  The walk still decides the cell: the
// prediction is only a starting cell (the learned walk in fdf_fp32.cu); inference runs on
// tcgen05 (fdf_mlp_tc.cu).
//
// A training step is two launches: k_train_tc carries each 128-sample tile of the minibatch
// through the forward, the loss and the backward on the 5th-generation tensor cores
// (tcgen05.mma, kind::f16, bfloat16 operands, FP32 accumulators in tensor memory) and writes the
// tile's gradient partials; k_train_update adds the partials in tile order and takes the Adam
// step on the FP32 master weights.  Every sum runs in a fixed order, so training is
// deterministic.
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

// SiLU and its derivative in FP32 (training): s = sigmoid(z) from the fast exponential and
// division intrinsics (s -> 0 as z -> -inf: 1 / (1 + inf) is 0), SiLU = z s,
// SiLU' = s (1 + z (1 - s)).
__device__ __forceinline__ float sigmoid_f(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid_f(z); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = sigmoid_f(z);
  return s * (1.0f + z * (1.0f - s));
}

// Polls of an mbarrier before a tensor-core wait is given up.
constexpr unsigned long long GT_WAIT_LIMIT = 1ull << 22;

// ---------------------------------------------------------------- training elementwise
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
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

// ---------------------------------------------------------------- fused training step
// One CTA carries a tile of 128 samples through the whole step on tcgen05: the forward
// (four layers), the loss and its gradient, and the backward (dH and dW of every layer), with
// the weights' bfloat16 image, the tile's inputs, one activation buffer and one gradient buffer
// in shared memory, and the pre-activations C1..C3 (FP32, bias not yet added) kept in tensor
// memory for the SiLU derivative.  Every operand is stored once, K-major by sample row; the
// products that need it transposed (dH = G W reads W, dW = G^T H reads G and H with the sample
// as K) read it MN-major.  Activations are rounded as the unfused step rounds them (bfloat16
// operands, FP32 accumulators, FP32 bias add, SiLU and SiLU' in FP32); H1 and H2 are recomputed
// from C1 and C2 for the backward instead of being kept.
//
// Sample row r of the tile is TMEM lane r; its four threads (warps w, w + 4, w + 8, w + 12 share
// the lane quarter of w % 4) take accumulator columns 0-31, 32-63, 64-95 and 96-127.  The tile's gradient partials
// (dW of its rows, bias sums, loss) go to part [tile][MLP_PART_STRIDE] in the parameter layout;
// k_train_update adds them in tile order, so the result does not depend on scheduling.
//
// Tensor memory: C1 columns 0-127, C2 128-255, C3 256-383, working accumulator 384-511; the
// dH of a layer lands in the columns of the C it no longer needs.  Every wait is bounded: past
// the limit the CTA records ERRBIT_TC_TIMEOUT, frees its tensor memory and returns.
constexpr int TT_THREADS = 512;
constexpr unsigned TT_SM_X = MLP_IMG_BYTES;          // [128][16]  inputs' bfloat16 pairs
constexpr unsigned TT_SM_H = TT_SM_X + 4096;         // [128][128] activations of one layer
constexpr unsigned TT_SM_G = TT_SM_H + 32768;        // [128][128] gradient of a hidden layer's output
constexpr unsigned TT_SM_G4 = TT_SM_G + 32768;       // [128][16]  gradient of the network's output
constexpr unsigned TT_SM_RED = TT_SM_G4 + 4096;      // [4][128]   per-warp column sums (bias gradients)
constexpr unsigned TT_SM_BIAS = TT_SM_RED + 2048;    // b1 | b2 | b3 | b4 in FP32 (387, padded)
constexpr unsigned TT_SM_LOSS = TT_SM_BIAS + 1600;   // [4] per-warp loss sums
constexpr unsigned TT_SM_BAR = TT_SM_LOSS + 32;      // mbarrier (8 B), TMEM base (4 B), time-out flag (4 B)
constexpr unsigned TT_SM_END = TT_SM_BAR + 16;
// The allocation, more than half an SM's shared memory, keeps one CTA per SM: the CTA takes all
// 512 TMEM columns, so a second one would wait in its allocation.
constexpr unsigned TT_SM_LAUNCH = 192 * 1024;
static_assert(TT_SM_END <= TT_SM_LAUNCH && TT_SM_LAUNCH > 114 * 1024, "training step shared memory");
constexpr unsigned TT_C1 = 0, TT_C2 = 128, TT_C3 = 256, TT_D = 384;
// The MN-major (transposed) reading of an operand stored K-major with 8-row groups sbo bytes
// apart: the leading byte offset is sbo (the stored rows are its K), the stride byte offset 128
// (the stored columns, 8 to a core-matrix row, are its M or N).
__device__ __forceinline__ unsigned long long mn_desc(unsigned addr, unsigned sbo) {
  return fdftc::make_desc(addr, sbo, 128);
}

// Column sums over the warp's 32 rows of 16 values per lane (a reduce-scatter: each exchange
// halves the values a lane keeps).  Returns, in every lane, the warp's sum of column
// 8 b4 + 4 b3 + 2 b2 + b1 (b_k: bit k of the lane); the order of the additions is fixed.
__device__ __forceinline__ float warp_colsum16(float (&v)[16], int lane) {
#pragma unroll
  for (int o = 16, h = 8; o >= 2; o >>= 1, h >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q < h) {
        const float send = up ? v[q] : v[q + h];
        const float keep = up ? v[q + h] : v[q];
        v[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
  }
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}
__device__ __forceinline__ int colsum16_column(int lane) {
  return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
}

__device__ __forceinline__ unsigned bf16x2(float lo, float hi) {
  unsigned v;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v) : "f"(hi), "f"(lo));
  return v;
}

__global__ void __launch_bounds__(TT_THREADS, 1)
    k_train_tc(const unsigned char *__restrict__ wimg, const float *__restrict__ params, const float *__restrict__ xs,
               const float *__restrict__ ts, long long n_samples, unsigned long long seed, long long step,
               int hashed, int B, float sx, float sy, float sz, float *__restrict__ part,
               float *__restrict__ loss_part, unsigned int *__restrict__ err, unsigned long long wait_limit,
               int stall_test) {
  using namespace fdftc;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, cg = warp >> 2;   // lane quarter, column group
  const int row = 32 * quarter + lane;                       // sample row = TMEM lane
  const unsigned lane_base = (unsigned)(32 * quarter) << 16;
  const long long tile = blockIdx.x;
  const long long b = tile * 128 + row;
  const bool valid = b < (long long)B;
  float *bias = reinterpret_cast<float *>(smem + TT_SM_BIAS);
  float *red = reinterpret_cast<float *>(smem + TT_SM_RED);
  float *lsum = reinterpret_cast<float *>(smem + TT_SM_LOSS);
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(smem + TT_SM_BAR + 8);
  volatile unsigned *tflag = reinterpret_cast<volatile unsigned *>(smem + TT_SM_BAR + 12);
  const unsigned bar = smem_u32(smem + TT_SM_BAR), sb = smem_u32(smem);
  float *prt = part + tile * MLP_PART_STRIDE;
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(wimg);
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int q = tid; q < MLP_IMG_BYTES / 16; q += TT_THREADS) dst[q] = src[q];
    for (int q = tid; q < 387; q += TT_THREADS)
      bias[q] = params[q < 128 ? MLP_OFF_B1 + q : q < 256 ? MLP_OFF_B2 + q - 128 : q < 384 ? MLP_OFF_B3 + q - 256
                                                                                       : MLP_OFF_B4 + q - 384];
  }
  float tgt[3] = {0.f, 0.f, 0.f};
  if (cg == 0) {   // the sample: X row [hi x, y, z, lo x, y, z, 0, ...], its target in registers
    float x[3] = {0.f, 0.f, 0.f};
    if (valid) {
      long long si = b;
      if (hashed) {
        const unsigned long long h = mix64(mix64(seed * 0xD1B54A32D192ED03ULL + (unsigned long long)step) +
                                           (unsigned long long)b * 0x9E3779B97F4A7C15ULL);
        si = (long long)(h % (unsigned long long)n_samples);
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) { x[d] = xs[3 * si + d]; tgt[d] = ts[3 * si + d]; }
    }
    float hi[3], lo[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      hi[d] = __bfloat162float(__float2bfloat16_rn(x[d]));
      lo[d] = x[d] - hi[d];
    }
    *reinterpret_cast<uint4 *>(smem + TT_SM_X + op_off(row, 0, 256)) =
        make_uint4(bf16x2(hi[0], hi[1]), bf16x2(hi[2], lo[0]), bf16x2(lo[1], lo[2]), 0u);
    *reinterpret_cast<uint4 *>(smem + TT_SM_X + op_off(row, 8, 256)) = make_uint4(0u, 0u, 0u, 0u);
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *tflag = 0u;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const unsigned tmem = *tmem_slot;
  const unsigned tl = tmem + lane_base;   // this thread's lane in every column
  unsigned phase = 0;

  // the stores of this step become visible to the tensor core, then one thread issues
  auto sync_issue = [&]() {
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
  };
  // waits for the last commit; all threads agree on a time-out
  auto wait_mma = [&]() -> bool {
    bool done = false;
    for (unsigned long long it = 0; it < wait_limit && !done; ++it) done = mbar_try_wait(bar, phase);
    phase ^= 1u;
    if (!done) *tflag = 1u;
    __syncthreads();
    const bool ok = *tflag == 0u;
    fence_after_sync();
    return ok;
  };
  // K-major operand of K columns (sbo = 16 K), K steps of 16 at 256 B
  auto gemm_kk = [&](unsigned d, unsigned a, unsigned a_sbo, unsigned bb, unsigned b_sbo, unsigned id, int ks) {
    for (int k = 0; k < ks; ++k)
      mma_f16(d, make_desc(a + 256u * k, 128, a_sbo), make_desc(bb + 256u * k, 128, b_sbo), id, k > 0 ? 1u : 0u);
  };
  // hidden-layer epilogue: H = bf16(SiLU(C + b)) into the activation buffer
  auto epi_hidden = [&](unsigned cc, const float *bl) {
#pragma unroll 1
    for (int c = 0; c < 2; ++c) {
      const int col = 32 * cg + 16 * c;
      float v[16];
      tmem_ld16(tl + cc + (unsigned)col, v);
      unsigned w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) w[q] = bf16x2(silu(v[2 * q] + bl[col + 2 * q]), silu(v[2 * q + 1] + bl[col + 2 * q + 1]));
      *reinterpret_cast<uint4 *>(smem + TT_SM_H + op_off(row, col, 2048)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4 *>(smem + TT_SM_H + op_off(row, col + 8, 2048)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
  };
  // backward epilogue: G = dH * SiLU'(C + b) (FP32) into the gradient buffer as bfloat16, and
  // the warp's column sums of G into red[quarter][column]
  auto epi_back = [&](unsigned dc, unsigned cc, const float *bl) {
#pragma unroll 1
    for (int c = 0; c < 2; ++c) {
      const int col = 32 * cg + 16 * c;
      float dv[16], zv[16];
      tmem_ld16(tl + dc + (unsigned)col, dv);
      tmem_ld16(tl + cc + (unsigned)col, zv);
      float g[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) g[q] = dv[q] * silu_grad(zv[q] + bl[col + q]);
      unsigned w[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) w[q] = bf16x2(g[2 * q], g[2 * q + 1]);
      *reinterpret_cast<uint4 *>(smem + TT_SM_G + op_off(row, col, 2048)) = make_uint4(w[0], w[1], w[2], w[3]);
      *reinterpret_cast<uint4 *>(smem + TT_SM_G + op_off(row, col + 8, 2048)) = make_uint4(w[4], w[5], w[6], w[7]);
      const float cs = warp_colsum16(g, lane);
      if ((lane & 1) == 0) red[quarter * 128 + col + colsum16_column(lane)] = cs;
    }
  };
  // this thread's 32 columns of a 128 x 128 dW in the working columns, as row `row` of W
  auto store_dw = [&](int off) {
#pragma unroll 1
    for (int c = 0; c < 2; ++c) {
      const int col = 32 * cg + 16 * c;
      float v[16];
      tmem_ld16(tl + TT_D + (unsigned)col, v);
      float4 *dst = reinterpret_cast<float4 *>(prt + off + row * 128 + col);
#pragma unroll
      for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
  };
  // bias gradient of a hidden layer: the four warps' column sums in fixed order
  auto store_db = [&](int off) {
    if (tid < 128) prt[off + tid] = ((red[tid] + red[128 + tid]) + red[256 + tid]) + red[384 + tid];
  };
  const unsigned id_h = make_idesc(128, 128, true), id_o = make_idesc(128, 16, true);
  const unsigned id_hh = make_idesc_t(128, 128, true, true, true);   // dW = G^T H
  const unsigned id_hb = make_idesc_t(128, 128, true, false, true);  // dH = G W
  const unsigned id_oo = make_idesc_t(128, 16, true, true, true);    // dW4^T = H3^T G4, dW1x = G1^T X
  const unsigned aX = sb + TT_SM_X, aH = sb + TT_SM_H, aG = sb + TT_SM_G, aG4 = sb + TT_SM_G4;
  bool ok = true;
  do {
    // ---- forward: C1 = X W1x^T, then C2, C3, and the output
    sync_issue();
    if (tid == 0 && !stall_test) {   // stall_test (tests of the time-out path only): nothing is
      fence_after_sync();            // issued or committed, so the first wait runs out
      gemm_kk(tmem + TT_C1, aX, 256, sb + MLP_IMG_W1, 256, id_h, 1);
      mma_commit(bar);
    }
    if (!(ok = wait_mma())) break;
    epi_hidden(TT_C1, bias);
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      gemm_kk(tmem + TT_C2, aH, 2048, sb + MLP_IMG_W2, 2048, id_h, 8);
      mma_commit(bar);
    }
    if (!(ok = wait_mma())) break;
    epi_hidden(TT_C2, bias + 128);
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      gemm_kk(tmem + TT_C3, aH, 2048, sb + MLP_IMG_W3, 2048, id_h, 8);
      mma_commit(bar);
    }
    if (!(ok = wait_mma())) break;
    epi_hidden(TT_C3, bias + 256);   // H3 stays in the activation buffer for dW4
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      gemm_kk(tmem + TT_D, aH, 2048, sb + MLP_IMG_W4, 2048, id_o, 8);
      mma_commit(bar);
    }
    if (!(ok = wait_mma())) break;
    // ---- output: y = C4 + b4, the loss and its gradient G4 = dloss/dy (FP32; bfloat16 operand)
    if (cg == 0) {
      float v[16];
      tmem_ld16(tl + TT_D, v);
      const float sc[3] = {sx, sy, sz};
      float g[3] = {0.f, 0.f, 0.f}, e2 = 0.f;
      if (valid) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float y = v[d] + bias[384 + d];
          const float e = (y - tgt[d]) * sc[d];
          e2 += e * e;
          g[d] = 2.0f * e * sc[d] / (3.0f * (float)B);
        }
      }
      *reinterpret_cast<uint4 *>(smem + TT_SM_G4 + op_off(row, 0, 256)) =
          make_uint4(bf16x2(g[0], g[1]), bf16x2(g[2], 0.f), 0u, 0u);
      *reinterpret_cast<uint4 *>(smem + TT_SM_G4 + op_off(row, 8, 256)) = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
#pragma unroll
        for (int d = 0; d < 3; ++d) g[d] += __shfl_xor_sync(0xffffffffu, g[d], o);
      }
      if (lane == 0) {
        lsum[quarter] = e2;
#pragma unroll
        for (int d = 0; d < 3; ++d) red[quarter * 128 + d] = g[d];
      }
    }
    // ---- dW4^T = H3^T G4 (rows: H3's columns; K: the samples)
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_D, mn_desc(aH + 4096u * k, 2048), mn_desc(aG4 + 512u * k, 256), id_oo, k > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    if (tid < 3) prt[MLP_OFF_B4 + tid] = ((red[tid] + red[128 + tid]) + red[256 + tid]) + red[384 + tid];
    if (tid == 3) loss_part[tile] = (((lsum[0] + lsum[1]) + lsum[2]) + lsum[3]) / (3.0f * (float)B);
    if (!(ok = wait_mma())) break;
    if (cg == 0) {
      float v[16];
      tmem_ld16(tl + TT_D, v);
#pragma unroll
      for (int o = 0; o < 3; ++o) prt[MLP_OFF_W4 + o * 128 + row] = v[o];
    }
    // ---- dH3 = G4 W4 into the working columns
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      mma_f16(tmem + TT_D, make_desc(aG4, 128, 256), mn_desc(sb + MLP_IMG_W4, 2048), id_hb, 0u);
      mma_commit(bar);
    }
    if (!(ok = wait_mma())) break;
    epi_back(TT_D, TT_C3, bias + 256);   // G3
    epi_hidden(TT_C2, bias + 128);      // H2 again
    // ---- dW3 = G3^T H2 (working columns), dH2 = G3 W3 (C3's columns)
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_D, mn_desc(aG + 4096u * k, 2048), mn_desc(aH + 4096u * k, 2048), id_hh, k > 0 ? 1u : 0u);
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_C3, make_desc(aG + 256u * k, 128, 2048), mn_desc(sb + MLP_IMG_W3 + 4096u * k, 2048), id_hb,
                k > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    store_db(MLP_OFF_B3);
    if (!(ok = wait_mma())) break;
    store_dw(MLP_OFF_W3);
    epi_back(TT_C3, TT_C2, bias + 128);   // G2
    epi_hidden(TT_C1, bias);             // H1 again
    // ---- dW2 = G2^T H1 (working columns), dH1 = G2 W2 (C2's columns)
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_D, mn_desc(aG + 4096u * k, 2048), mn_desc(aH + 4096u * k, 2048), id_hh, k > 0 ? 1u : 0u);
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_C2, make_desc(aG + 256u * k, 128, 2048), mn_desc(sb + MLP_IMG_W2 + 4096u * k, 2048), id_hb,
                k > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    store_db(MLP_OFF_B2);
    if (!(ok = wait_mma())) break;
    store_dw(MLP_OFF_W2);
    epi_back(TT_C2, TT_C1, bias);   // G1
    // ---- dW1x = G1^T X: the W1 gradient is the sum of its two column groups (hi and lo inputs)
    sync_issue();
    if (tid == 0) {
      fence_after_sync();
      for (int k = 0; k < 8; ++k)
        mma_f16(tmem + TT_D, mn_desc(aG + 4096u * k, 2048), mn_desc(aX + 512u * k, 256), id_oo, k > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    store_db(MLP_OFF_B1);
    if (!(ok = wait_mma())) break;
    if (cg == 0) {
      float v[16];
      tmem_ld16(tl + TT_D, v);
#pragma unroll
      for (int d = 0; d < 3; ++d) prt[MLP_OFF_W1 + row * 3 + d] = v[d] + v[3 + d];
    }
  } while (false);
  if (!ok && tid == 0) atomicOr(err, (unsigned)ERRBIT_TC_TIMEOUT);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512) : "memory");
  }
}

// grads = the tiles' partials added in tile order; with adam, the Adam step (as k_adam) on the
// FP32 parameters and their bfloat16 image rewritten for the next step.
__global__ void k_train_update(const float *__restrict__ part, int tiles, const float *__restrict__ loss_part,
                               float *__restrict__ params, float *__restrict__ grads, float *__restrict__ m,
                               float *__restrict__ v, unsigned char *__restrict__ wimg, float *__restrict__ loss_out,
                               int adam, float lr, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0 && loss_out) {
    float l = 0.f;
    for (int t = 0; t < tiles; ++t) l += loss_part[t];
    *loss_out = l;
  }
  if (q >= MLP_NPARAM) return;
  float g = 0.f;
  for (int t = 0; t < tiles; ++t) g += part[(long long)t * MLP_PART_STRIDE + q];
  grads[q] = g;
  if (!adam) return;
  const float mq = 0.9f * m[q] + 0.1f * g;
  const float vq = 0.999f * v[q] + 0.001f * g * g;
  m[q] = mq;
  v[q] = vq;
  const float w = params[q] - lr * (mq / c1) / (sqrtf(vq / c2) + 1e-8f);
  params[q] = w;
  const __nv_bfloat16 wb = __float2bfloat16_rn(w);
  const unsigned short bits = *reinterpret_cast<const unsigned short *>(&wb);
  unsigned short *img = reinterpret_cast<unsigned short *>(wimg);
  using fdftc::op_off;
  if (q < MLP_OFF_B1) {   // W1 [128][3]: columns k and k + 3 of the image (the inputs' hi and lo parts)
    const int n = q / 3, k = q % 3;
    img[(MLP_IMG_W1 + op_off(n, k, 256)) / 2] = bits;
    img[(MLP_IMG_W1 + op_off(n, k + 3, 256)) / 2] = bits;
  } else if (q >= MLP_OFF_W2 && q < MLP_OFF_B2) {
    const int o = q - MLP_OFF_W2;
    img[(MLP_IMG_W2 + op_off(o / 128, o % 128, 2048)) / 2] = bits;
  } else if (q >= MLP_OFF_W3 && q < MLP_OFF_B3) {
    const int o = q - MLP_OFF_W3;
    img[(MLP_IMG_W3 + op_off(o / 128, o % 128, 2048)) / 2] = bits;
  } else if (q >= MLP_OFF_W4 && q < MLP_OFF_B4) {
    const int o = q - MLP_OFF_W4;
    img[(MLP_IMG_W4 + op_off(o / 128, o % 128, 2048)) / 2] = bits;
  }
}

inline unsigned blocks_for(long long n, int th) { return (unsigned)(n > 0 ? (n + th - 1) / th : 1); }

}  // namespace

// ---------------------------------------------------------------- host side
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

void mlp_train_step(const unsigned char *wimg, const float *params, const float *xs, const float *ts,
                    long long n_samples, unsigned long long seed, long long step, int hashed, int B,
                    const float sc[3], float *part, float *loss_part, unsigned int *err, cudaStream_t s,
                    int stall_test) {
  static int attr_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (attr_device != dev) {
    cudaFuncSetAttribute(k_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TT_SM_LAUNCH);
    attr_device = dev;
  }
  k_train_tc<<<(unsigned)mlp_train_tiles(B), TT_THREADS, TT_SM_LAUNCH, s>>>(
      wimg, params, xs, ts, n_samples, seed, step, hashed, B, sc[0], sc[1], sc[2], part, loss_part, err,
      stall_test ? 1024ull : GT_WAIT_LIMIT, stall_test);
}
void mlp_train_update(const float *part, int tiles, const float *loss_part, float *params, float *grads, float *m,
                      float *v, unsigned char *wimg, float *loss_out, int adam, float lr, float c1, float c2,
                      cudaStream_t s) {
  k_train_update<<<blocks_for(MLP_NPARAM, 256), 256, 0, s>>>(part, tiles, loss_part, params, grads, m, v, wimg,
                                                             loss_out, adam, lr, c1, c2);
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
