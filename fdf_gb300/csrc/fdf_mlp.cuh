// fdf_mlp.cuh -- layout and launchers of the learned start-cell locator (fdf_mlp.cu).
//
// Parameters, FP32 master copy, one contiguous vector (row-major W [out][in]):
//   W1 [128][3] | b1 [128] | W2 [128][128] | b2 [128] | W3 [128][128] | b3 [128] | W4 [3][128] | b4 [3]
// Inference weights: the tcgen05 kernel's shared-memory image (fdf_mlp_tc.cu, bfloat16 or half
// precision) and the biases.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "fdf_internal.cuh"

#define MLP_H 128
#define MLP_OFF_W1 0
#define MLP_OFF_B1 384
#define MLP_OFF_W2 512
#define MLP_OFF_B2 16896
#define MLP_OFF_W3 17024
#define MLP_OFF_B3 33408
#define MLP_OFF_W4 33536
#define MLP_OFF_B4 33920
#define MLP_NPARAM 33923

#define MLP_BIAS_WORDS 392      // b1/2 | b2/2 | b3/2 | b4 (387 used; hidden biases halved for the SiLU epilogue)

// Input normalisation xhat = (x - centre) * inv_half, in FP32.
struct MlpNorm {
  float centre[3];
  float inv_half[3];
};

// Training building blocks (all on stream s, deterministic).  mlp_gemm runs on tcgen05 and sets
// ERRBIT_TC_TIMEOUT in *err if a tensor-core wait runs out.  X rows are the inputs' bfloat16
// pairs [hi x, y, z, lo x, y, z] (mlp_split_inputs), multiplied by W1x = [W1 | W1]
// (mlp_split_w1); mlp_fold_w1 adds the two column groups of the W1x gradient.
void mlp_gemm(const __nv_bfloat16 *A, long long sam, long long sak, const __nv_bfloat16 *B, long long sbk,
              long long sbn, float *C, long long scm, long long scn, int M, int N, int K, int splits,
              float *partials, unsigned int *err, cudaStream_t s);
void mlp_gather_batch(const float *xs, const float *ts, long long n_samples, unsigned long long seed, long long step,
                      int B, __nv_bfloat16 *X, float *T, cudaStream_t s);
void mlp_split_inputs(const float *xs, int B, __nv_bfloat16 *X, cudaStream_t s);
void mlp_split_w1(const __nv_bfloat16 *w1, __nv_bfloat16 *w1x, cudaStream_t s);
void mlp_fold_w1(const float *dw1x, float *dw1, cudaStream_t s);
void mlp_bias_silu(const float *C, const float *b, int B, int N, float *Z, __nv_bfloat16 *H, cudaStream_t s);
void mlp_out_loss(const float *C4, const float *b4, const float *T, int B, const float sc[3], float *Y, float *G,
                  __nv_bfloat16 *Gb, float *loss_part, cudaStream_t s);
void mlp_silu_bwd(const float *dH, const float *Z, long long total, float *G, __nv_bfloat16 *Gb, cudaStream_t s);
void mlp_colsum(const float *G, int B, int N, float *db, cudaStream_t s);
void mlp_adam(float *w, const float *g, float *m, float *v, int n, float lr, float c1, float c2, cudaStream_t s);
void mlp_to_bf16(const float *in, __nv_bfloat16 *out, int n, cudaStream_t s);
void mlp_sum_partials(const float *part, int n, float *out, cudaStream_t s);
void mlp_pack_bias(const float *params, float *bias, cudaStream_t s);

// Training samples from located points: xs = normalised FP32 position, ts = cell-centre target.
// keep[s] != 0 marks a located point; slot[s] = its exclusive-scan position.
void mlp_make_samples(const double *x, const double *y, const double *z, const int *cell, const unsigned int *slot,
                      const unsigned int *keep, long long n, MlpNorm norm, GridDims g, float *xs, float *ts,
                      cudaStream_t s);
void mlp_flag_located(const int *cell, const unsigned char *status, long long n, unsigned int *flag, cudaStream_t s);

// Initial weights: W uniform in +-1/sqrt(fan_in) from the splitmix64 streams (seed, 100 + layer),
// biases zero (host).
void mlp_init_params_host(unsigned long long seed, float *params);

// Inference on tcgen05 (fdf_mlp_tc.cu): guess[t] = predicted cell of particle list[t]
// (t < *list_count), positions read as float pairs (hi, lo) from the precision-form swarm
// arrays; list == nullptr: particles 0 .. n_host-1, positions read as FP64 from x, y, z.
// yout (optional): the network's outputs [n][3].  The weights are packed once into the CTA's
// shared-memory image (mlp_tc_image_bytes() bytes), bfloat16 (bf16 != 0) or half precision;
// the image and the launch must agree.  A timed-out tensor-core wait sets ERRBIT_TC_TIMEOUT in
// *err.  stall_test != 0 is for tests of that path: the kernel issues no MMA, so its first
// bounded wait (1024 polls) runs out and the CTAs return with the error bit.
size_t mlp_tc_image_bytes();
void mlp_pack_tc(const float *params, unsigned char *img, int bf16, cudaStream_t s);
void mlp_guess_tc(const unsigned char *img, int bf16, const float *bias, const MlpNorm &norm, const double *x,
                  const double *y, const double *z, int pairs, const unsigned int *list,
                  const unsigned long long *list_count, int n_host, int n_cap, GridDims g, int *guess, int num_sms,
                  unsigned int *err, cudaStream_t s, float *yout = nullptr, int stall_test = 0);
