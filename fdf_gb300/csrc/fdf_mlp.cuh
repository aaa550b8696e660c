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

// The weights' shared-memory image (16-bit, K-major core-matrix layout of fdf_tc.cuh), shared by
// inference and training: W1 [128][16] (K padded from 3; the bfloat16 image repeats W1 in
// columns 3-5 for the inputs' low parts), W2 and W3 [128][128], W4 [16][128] (N padded from 3).
#define MLP_IMG_W1 0
#define MLP_IMG_W2 4096
#define MLP_IMG_W3 36864
#define MLP_IMG_W4 69632
#define MLP_IMG_BYTES 73728

// Per-tile gradient partials of the fused training step: one row of MLP_PART_STRIDE floats per
// 128-sample tile, in the parameter layout.
#define MLP_PART_STRIDE 33936

// Input normalisation xhat = (x - centre) * inv_half, in FP32.
struct MlpNorm {
  float centre[3];
  float inv_half[3];
};

void mlp_pack_bias(const float *params, float *bias, cudaStream_t s);

// Training samples from located points: xs = normalised FP32 position, ts = cell-centre target.
// keep[s] != 0 marks a located point; slot[s] = its exclusive-scan position.
void mlp_make_samples(const double *x, const double *y, const double *z, const int *cell, const unsigned int *slot,
                      const unsigned int *keep, long long n, MlpNorm norm, GridDims g, float *xs, float *ts,
                      cudaStream_t s);
void mlp_flag_located(const int *cell, const unsigned char *status, long long n, unsigned int *flag, cudaStream_t s);

// Fused training step on tcgen05 (fdf_mlp.cu): the loss and gradients of a batch of B samples,
// one CTA per 128-sample tile.  Sample b of the batch is xs/ts row mix64(seed, step, b) mod n
// (hashed != 0, the training minibatch) or row b (hashed == 0).  wimg is the bfloat16 image of
// the current weights, params the FP32 parameters (the biases are read from there).  Each tile
// writes its gradient partials to part [tiles][MLP_PART_STRIDE] and its share of the loss to
// loss_part [tiles].  mlp_train_update then adds the partials in tile order into grads (and the
// loss into *loss_out), and with adam != 0 takes the Adam step on params and rewrites wimg.  A
// timed-out tensor-core wait sets ERRBIT_TC_TIMEOUT in *err; stall_test != 0 is for tests of that
// path: no MMA is issued, so each CTA's first bounded wait (1024 polls) runs out.
void mlp_train_step(const unsigned char *wimg, const float *params, const float *xs, const float *ts,
                    long long n_samples, unsigned long long seed, long long step, int hashed, int B,
                    const float sc[3], float *part, float *loss_part, unsigned int *err, cudaStream_t s,
                    int stall_test = 0);
void mlp_train_update(const float *part, int tiles, const float *loss_part, float *params, float *grads, float *m,
                      float *v, unsigned char *wimg, float *loss_out, int adam, float lr, float c1, float c2,
                      cudaStream_t s);
inline int mlp_train_tiles(int B) { return (B + 127) / 128; }

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
