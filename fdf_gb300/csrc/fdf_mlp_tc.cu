// fdf_mlp_tc.cu -- inference of the learned start-cell locator on the 5th-generation tensor
// cores (tcgen05): one CTA holds the network's weights in shared memory as 16-bit values
// (bfloat16 by default, as the network trains; half precision on request) and carries tiles
// of 128 particles through the four layers; each layer is tcgen05.mma (M = 128, kind::f16,
// 16-bit operands from shared memory, FP32 accumulator in tensor memory), issued by one thread
// and tracked by an mbarrier; the four warps then read the accumulator rows back with
// tcgen05.ld (one particle per thread), add the bias, apply SiLU in packed 16-bit pair
// arithmetic and store the activations as the next layer's A operand.  One CTA per SM holds
// the weights once and runs four independent tile pipelines (one per warpgroup, each with its
// own activation buffers, mbarrier and 128 TMEM columns), so the tensor core serves one
// pipeline's MMAs while the others run their epilogues.  Each epilogue reads the accumulator 32
// columns at a time with the next 32 in flight, and each pipeline loads its next tile's particle
// indices and positions one layer before it uses them, so neither latency stalls the chain.
//
// Input layer.  A bfloat16 coordinate carries 8 significant bits, coarser than a cell of a
// long grid (1536 cells over the normalised range [-1, 1] are 0.0013 wide; bfloat16's spacing
// near 1 is 0.0078).  The bfloat16 form therefore feeds each normalised coordinate as a pair
// hi = bf16(x), lo = bf16(x - hi) (16 significant bits) in K columns 0-2 and 3-5 of the
// first layer, whose weight image repeats W1 in both column groups: W1 (hi + lo) is summed in
// the FP32 accumulator.  The half-precision form feeds x, y, z once (11 significant bits).
//
// Shared-memory operands use the K-major core-matrix layout of fdf_tc.cuh.
//
// Every wait on an mbarrier is bounded: past the limit the CTA records ERRBIT_TC_TIMEOUT,
// frees its tensor memory and returns.
#include "fdf_internal.cuh"
#include "fdf_mlp.cuh"
#include "fdf_tc.cuh"
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace {

using namespace fdftc;

constexpr int TC_ROWS = 128;                 // particles per tile (MMA M)
constexpr int TC_PIPES = 4;                  // warpgroups per CTA, one tile pipeline each
constexpr int TC_THREADS = 128 * TC_PIPES;
constexpr int TC_TMEM_COLS = 128 * TC_PIPES; // FP32 accumulator columns, 128 per pipeline
// shared memory map (bytes)
constexpr int SM_W1 = MLP_IMG_W1;            // [128][16]  4096
constexpr int SM_W2 = MLP_IMG_W2;            // [128][128] 32768
constexpr int SM_W3 = MLP_IMG_W3;            // [128][128] 32768
constexpr int SM_W4 = MLP_IMG_W4;            // [16][128]  4096
constexpr int SM_PIPE = MLP_IMG_BYTES;       // per pipeline: A1 [128][16] 4096, A [128][128] 32768
constexpr int PIPE_BYTES = 4096 + 32768;
constexpr int SM_BIAS = SM_PIPE + TC_PIPES * PIPE_BYTES;   // 392 floats
constexpr int SM_HB2 = SM_BIAS + 1568;       // the hidden half-biases as 192 16-bit pairs
constexpr int SM_BAR = SM_HB2 + 768;         // mbarriers (8 B each), TMEM base (4 B), time-out flags
constexpr int SM_TOTAL = SM_BAR + 8 * TC_PIPES + 8 + 4 * TC_PIPES;
constexpr int WIMG_BYTES = SM_PIPE;          // packed weight image in global memory (73,728 B)
constexpr unsigned long long WAIT_LIMIT = 1ull << 22;

// Two FP32 values rounded to a 16-bit pair, lo in the low half.
template <bool BF16>
__device__ __forceinline__ unsigned pack2(float lo, float hi) {
  unsigned v;
  if constexpr (BF16) asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v) : "f"(hi), "f"(lo));
  else asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(v) : "f"(hi), "f"(lo));
  return v;
}

// SiLU(z) = z * sigmoid(z) = h + h * tanh(h) with h = z / 2, on a pair of columns in packed
// 16-bit arithmetic: the accumulator pair v01 rounded to the operand type, h = v/2 + hb (hb:
// the half-bias pair), one tanh.approx of the pair, h + h t -- four instructions per pair.
// The epilogue is bound by instruction issue, so this halves its cost against the FP32 form
// of the same formula.  The pair is the next layer's A operand as it stands.
template <bool BF16>
__device__ __forceinline__ unsigned silu2(unsigned v01, unsigned hb) {
  unsigned h, t, s;
  if constexpr (BF16) {
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(h) : "r"(v01), "r"(0x3F003F00u), "r"(hb));   // 0.5 in both halves
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(s) : "r"(h), "r"(t), "r"(h));
  } else {
    asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(h) : "r"(v01), "r"(0x38003800u), "r"(hb));
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(h));
    asm("fma.rn.f16x2 %0, %1, %2, %3;" : "=r"(s) : "r"(h), "r"(t), "r"(h));
  }
  return s;
}

// Packs the FP32 parameters into the shared-memory image of the weights (bfloat16 or half
// precision); the bfloat16 image repeats W1 in K columns 3-5 for the inputs' low parts.
__global__ void k_pack_tc(const float *__restrict__ params, unsigned char *__restrict__ img, int bf16) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;   // one 16-bit element of the image
  if (q >= WIMG_BYTES / 2) return;
  const int byte = 2 * q;
  float v = 0.f;
  if (byte < SM_W2) {                                   // W1 [128][16], K padded from 3 (or 6)
    const int o = byte - SM_W1;
    const int rg = o / 256, kc = (o % 256) / 128, rr = (o % 128) / 16, kk = (o % 16) / 2;
    const int n = rg * 8 + rr, k = kc * 8 + kk;
    if (k < 3) v = params[MLP_OFF_W1 + n * 3 + k];
    else if (bf16 && k < 6) v = params[MLP_OFF_W1 + n * 3 + k - 3];
  } else if (byte < SM_W4) {                            // W2, W3 [128][128]
    const bool second = byte >= SM_W3;
    const int o = byte - (second ? SM_W3 : SM_W2);
    const int rg = o / 2048, kc = (o % 2048) / 128, rr = (o % 128) / 16, kk = (o % 16) / 2;
    const int n = rg * 8 + rr, k = kc * 8 + kk;
    v = params[(second ? MLP_OFF_W3 : MLP_OFF_W2) + n * 128 + k];
  } else {                                              // W4 [16][128], N padded from 3
    const int o = byte - SM_W4;
    const int rg = o / 2048, kc = (o % 2048) / 128, rr = (o % 128) / 16, kk = (o % 16) / 2;
    const int n = rg * 8 + rr, k = kc * 8 + kk;
    if (n < 3) v = params[MLP_OFF_W4 + n * 128 + k];
  }
  unsigned short bits;
  if (bf16) {
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    bits = *reinterpret_cast<const unsigned short *>(&b);
  } else {
    const __half h = __float2half_rn(v);
    bits = *reinterpret_cast<const unsigned short *>(&h);
  }
  reinterpret_cast<unsigned short *>(img)[q] = bits;
}

template <bool BF16>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_mlp_guess_tc(const unsigned char *__restrict__ wimg, const float *__restrict__ bias_g, MlpNorm norm,
                   const double *__restrict__ px, const double *__restrict__ py, const double *__restrict__ pz,
                   int pairs, const unsigned int *__restrict__ list, const unsigned long long *__restrict__ list_count,
                   int n_host, GridDims g, int *__restrict__ guess, float *__restrict__ yout,
                   unsigned int *__restrict__ err, unsigned long long wait_limit, int stall_test) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int pipe = tid >> 7, row = tid & 127;     // warpgroup = pipeline; thread = tile row
  float *bias = reinterpret_cast<float *>(smem + SM_BIAS);
  unsigned *hb2 = reinterpret_cast<unsigned *>(smem + SM_HB2);
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + SM_BAR);
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(smem + SM_BAR + 8 * TC_PIPES);
  volatile unsigned *tflag = reinterpret_cast<volatile unsigned *>(smem + SM_BAR + 8 * TC_PIPES + 8);
  unsigned char *a1s = smem + SM_PIPE + pipe * PIPE_BYTES, *as = a1s + 4096;
  // weights and biases, once per CTA
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(wimg);
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int q = tid; q < WIMG_BYTES / 16; q += TC_THREADS) dst[q] = src[q];
    for (int q = tid; q < MLP_BIAS_WORDS; q += TC_THREADS) bias[q] = bias_g[q];
    for (int q = tid; q < 192; q += TC_THREADS) hb2[q] = pack2<BF16>(bias_g[2 * q], bias_g[2 * q + 1]);
    uint4 *a1 = reinterpret_cast<uint4 *>(a1s);
    for (int q = row; q < 4096 / 16; q += 128) a1[q] = make_uint4(0, 0, 0, 0);
  }
  const unsigned bar_addr = smem_u32(bars + pipe);
  if (row == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_addr) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    tflag[pipe] = 0u;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  // this pipeline's accumulator columns; this warp's TMEM lane quarter
  const unsigned tmem = *tmem_slot + (unsigned)(128 * pipe);
  const unsigned lane_base = (unsigned)((warp & 3) * 32) << 16;
  const unsigned sbase = smem_u32(smem), a1_addr = smem_u32(a1s), a_addr = smem_u32(as);
  const unsigned id_hidden = make_idesc(TC_ROWS, 128, BF16), id_out = make_idesc(TC_ROWS, 16, BF16);
  const unsigned pipe_bar = 1 + pipe;   // named barrier of this warpgroup (0 is __syncthreads)

  const long long n = list_count ? (long long)*list_count : (long long)n_host;
  const long long ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  const long long tile0 = (long long)blockIdx.x * TC_PIPES + pipe, tstride = (long long)gridDim.x * TC_PIPES;
  unsigned phase = 0;
  bool timed_out = false;

  auto pipe_sync = [&]() { asm volatile("bar.sync %0, 128;\n" ::"r"(pipe_bar) : "memory"); };
  // waits for the MMAs this pipeline committed last; its 128 threads agree on a time-out
  // (only the pipeline's first warp polls: the others wait at the named barrier, which issues
  // nothing, so the other pipelines' epilogues keep the schedulers)
  auto wait_mma = [&]() -> bool {
    if (row < 32) {
      bool done = false;
      for (unsigned long long it = 0; it < wait_limit && !done; ++it) done = mbar_try_wait(bar_addr, phase);
      if (!done) tflag[pipe] = 1u;
    }
    phase ^= 1u;
    pipe_sync();
    const bool bad = tflag[pipe] != 0u;
    fence_after_sync();
    return !bad;
  };
  // bias + SiLU of the 128 accumulator columns (b: half-biases), stored as the next layer's A operand,
  // 32 columns at a time (the next 32 columns' TMEM load is in flight while a chunk is converted)
  auto chunk = [&](const unsigned (&r)[32], const unsigned *b, int c) {
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      unsigned w[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int pq = 4 * h + q;   // column pair within the chunk
        w[q] = silu2<BF16>(pack2<BF16>(__uint_as_float(r[2 * pq]), __uint_as_float(r[2 * pq + 1])), b[16 * c + pq]);
      }
      *reinterpret_cast<uint4 *>(as + op_off(row, 32 * c + 8 * h, 2048)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  };
  auto epilogue = [&](const unsigned *b) {
    unsigned ra[32], rb[32];
    tmem_ld32_issue(tmem + lane_base, ra);
    tmem_wait_ld32(ra);
    tmem_ld32_issue(tmem + lane_base + 32u, rb);
    chunk(ra, b, 0);
    tmem_wait_ld32(rb);
    tmem_ld32_issue(tmem + lane_base + 64u, ra);
    chunk(rb, b, 1);
    tmem_wait_ld32(ra);
    tmem_ld32_issue(tmem + lane_base + 96u, rb);
    chunk(ra, b, 2);
    tmem_wait_ld32(rb);
    chunk(rb, b, 3);
  };
  // the next tile's inputs in two steps whose loads are consumed one layer later: its particle
  // index, then the raw 8-byte coordinates (an FP64 value, or a float pair (hi, lo))
  constexpr unsigned NO_ROW = 0xffffffffu;
  auto fetch_index = [&](long long tile) -> unsigned {
    const long long r = tile * TC_ROWS + row;
    if (tile >= ntiles || r >= n) return NO_ROW;
    return list ? list[r] : (unsigned int)r;
  };
  auto fetch_raw = [&](unsigned p, unsigned long long (&raw)[3]) {
    raw[0] = raw[1] = raw[2] = 0ull;
    if (p != NO_ROW) {
      raw[0] = reinterpret_cast<const unsigned long long *>(px)[p];
      raw[1] = reinterpret_cast<const unsigned long long *>(py)[p];
      raw[2] = reinterpret_cast<const unsigned long long *>(pz)[p];
    }
  };
  auto to_inputs = [&](unsigned p, const unsigned long long (&raw)[3], float &x, float &y, float &z) {
    float c[3] = {0.f, 0.f, 0.f};
    if (p != NO_ROW) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float v = pairs ? __int_as_float((int)(unsigned)(raw[d] & 0xffffffffull)) +
                                    __int_as_float((int)(unsigned)(raw[d] >> 32))
                              : (float)__longlong_as_double((long long)raw[d]);
        c[d] = (v - norm.centre[d]) * norm.inv_half[d];
      }
    }
    x = c[0]; y = c[1]; z = c[2];
  };
  // the MMAs of one layer, issued by the pipeline's first thread after its threads' stores
  auto issue = [&](int layer) {
    fence_async_smem();
    fence_before_sync();
    pipe_sync();
    if (row == 0) {
      fence_after_sync();
      if (layer == 0) {
        mma_f16(tmem, make_desc(a1_addr, 128, 256), make_desc(sbase + SM_W1, 128, 256), id_hidden, 0u);
      } else {
        const unsigned wb = layer == 1 ? SM_W2 : layer == 2 ? SM_W3 : SM_W4;
        const unsigned id = layer == 3 ? id_out : id_hidden;
#pragma unroll 1
        for (int k = 0; k < 8; ++k)
          mma_f16(tmem, make_desc(a_addr + 256 * k, 128, 2048), make_desc(sbase + wb + 256 * k, 128, 2048), id,
                  k > 0 ? 1u : 0u);
      }
      mma_commit(bar_addr);
    }
  };

  float cx, cy, cz;
  {
    unsigned long long raw[3];
    const unsigned p0 = fetch_index(tile0);
    fetch_raw(p0, raw);
    to_inputs(p0, raw, cx, cy, cz);
  }
#pragma unroll 1
  for (long long tile = tile0; tile < ntiles; tile += tstride) {
    const long long r = tile * TC_ROWS + row;
    if constexpr (BF16) {   // hi parts in K columns 0-2, lo parts in 3-5
      const float hx = __bfloat162float(__float2bfloat16_rn(cx)), hy = __bfloat162float(__float2bfloat16_rn(cy)),
                  hz = __bfloat162float(__float2bfloat16_rn(cz));
      *reinterpret_cast<uint4 *>(a1s + op_off(row, 0, 256)) =
          make_uint4(pack2<true>(hx, hy), pack2<true>(hz, cx - hx), pack2<true>(cy - hy, cz - hz), 0u);
    } else {
      *reinterpret_cast<uint4 *>(a1s + op_off(row, 0, 256)) =
          make_uint4(pack2<false>(cx, cy), pack2<false>(cz, 0.f), 0u, 0u);
    }
    // stall_test (tests of the time-out path only): nothing is issued or committed, so the wait
    // below runs out with no MMA in flight
    if (!stall_test) issue(0);
    const unsigned np = fetch_index(tile + tstride);   // the next tile's rows, while this one computes
    if (!wait_mma()) { timed_out = true; break; }
    epilogue(hb2);
    issue(1);
    unsigned long long nraw[3];
    fetch_raw(np, nraw);
    if (!wait_mma()) { timed_out = true; break; }
    epilogue(hb2 + 64);
    issue(2);
    if (!wait_mma()) { timed_out = true; break; }
    epilogue(hb2 + 128);
    issue(3);
    if (!wait_mma()) { timed_out = true; break; }
    {
      float v[16];
      tmem_ld16(tmem + lane_base, v);
      if (r < n) {
        const float y0 = v[0] + bias[384], y1 = v[1] + bias[385], y2 = v[2] + bias[386];
        if (yout) { yout[3 * r] = y0; yout[3 * r + 1] = y1; yout[3 * r + 2] = y2; }
        const float ys[3] = {y0, y1, y2};
        const int N[3] = {g.IM, g.JM, g.KM};
        int idx[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float t = (ys[d] + 1.0f) * 0.5f * (float)N[d];
          idx[d] = (t == t) ? (int)fminf(fmaxf(floorf(t), 0.f), (float)(N[d] - 1)) : 0;
        }
        guess[r] = (idx[2] * g.JM + idx[1]) * g.IM + idx[0];
      }
    }
    to_inputs(np, nraw, cx, cy, cz);
    fence_before_sync();   // this tile's TMEM reads finish before the next tile's MMAs (ordered by issue(0))
  }
  if (timed_out && row == 0) atomicOr(err, (unsigned)ERRBIT_TC_TIMEOUT);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(*tmem_slot), "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

}  // namespace

size_t mlp_tc_image_bytes() { return WIMG_BYTES; }

void mlp_pack_tc(const float *params, unsigned char *img, int bf16, cudaStream_t s) {
  k_pack_tc<<<(WIMG_BYTES / 2 + 255) / 256, 256, 0, s>>>(params, img, bf16);
}

void mlp_guess_tc(const unsigned char *img, int bf16, const float *bias, const MlpNorm &norm, const double *x,
                  const double *y, const double *z, int pairs, const unsigned int *list,
                  const unsigned long long *list_count, int n_host, int n_cap, GridDims g, int *guess, int num_sms,
                  unsigned int *err, cudaStream_t s, float *yout, int stall_test) {
  static int attr_device = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (attr_device != dev) {
    cudaFuncSetAttribute(k_mlp_guess_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    cudaFuncSetAttribute(k_mlp_guess_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_TOTAL);
    attr_device = dev;
  }
  const long long tiles = ((long long)n_cap + TC_ROWS - 1) / TC_ROWS;
  long long blocks = (tiles + TC_PIPES - 1) / TC_PIPES;
  const long long cap_blocks = (long long)num_sms;
  if (blocks > cap_blocks) blocks = cap_blocks;
  if (blocks < 1) blocks = 1;
  const unsigned long long limit = stall_test ? 1024ull : WAIT_LIMIT;
  if (bf16)
    k_mlp_guess_tc<true><<<(unsigned)blocks, TC_THREADS, SM_TOTAL, s>>>(img, bias, norm, x, y, z, pairs, list,
                                                                        list_count, n_host, g, guess, yout, err,
                                                                        limit, stall_test);
  else
    k_mlp_guess_tc<false><<<(unsigned)blocks, TC_THREADS, SM_TOTAL, s>>>(img, bias, norm, x, y, z, pairs, list,
                                                                         list_count, n_host, g, guess, yout, err,
                                                                         limit, stall_test);
}
