// fdf_locator.cu -- C ABI of the learned start-cell locator (FDF_FORM_LEARNED_FP32):
// parameter set-up, training on location pairs produced by the walking search, gradients
// for checking, and inference.  No counterpart in the reference, which starts every walk
// in the particle's previous cell (walkingsearch.c:571-626, InitializeTraversalParameters).
//
// Training (all on the context stream, deterministic):
//   samples   n points seeded like the volumetric initialisation (random cell, random
//             logical coordinates), each located by the plain FP64 walk from its generating
//             cell; the located (position, cell) pairs become (xhat, target) in FP32
//   step t    two launches: k_train_tc (one CTA per 128-sample tile of the minibatch drawn by
//             counter hash: forward, loss and backward on tcgen05, the tile's gradient
//             partials) and k_train_update (partials added in tile order, Adam on the FP32
//             master weights, their bfloat16 image rewritten for the next step)
//   finally   weights packed into the tcgen05 inference kernel's shared-memory image
#include "fdf_context.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

// Training scratch for batches of up to B samples: the tiles' gradient partials and losses (and the
// batch's loss), the
// samples of an explicit batch (fdf_LocatorGradients) and the tensor-core time-out word.
struct TrainScratch {
  float *part, *loss_part, *xs, *ts;
  unsigned int *err;
};

size_t scratch_bytes(int B) {
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t tiles = (size_t)mlp_train_tiles(B);
  return up(4 * tiles * MLP_PART_STRIDE) + up(4 * (tiles + 1)) + 2 * up(12 * (size_t)B) + up(4);
}

TrainScratch carve_scratch(void *base, int B) {
  char *p = (char *)base;
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) / 256 * 256;
    return (void *)r;
  };
  const size_t tiles = (size_t)mlp_train_tiles(B);
  TrainScratch s{};
  s.part = (float *)take(4 * tiles * MLP_PART_STRIDE);
  s.loss_part = (float *)take(4 * (tiles + 1));   // the tiles' losses, then the batch's
  s.xs = (float *)take(12 * (size_t)B);
  s.ts = (float *)take(12 * (size_t)B);
  s.err = (unsigned int *)take(4);
  return s;
}

int alloc_params(FdfContext *ctx) {
  LocatorState &L = ctx->loc;
  if (L.params && L.grads && L.adam_m && L.adam_v && L.train_img && L.bias && L.tc_img) return FDF_SUCCESS;
  // all or none: a partial set left by a failed allocation is freed and made again
  L.has_params = false;
  cfree(L.params); cfree(L.grads); cfree(L.adam_m); cfree(L.adam_v); cfree(L.train_img);
  cfree(L.bias); cfree(L.tc_img);
  CU(dev_alloc(&L.params, 4ull * MLP_NPARAM));
  CU(dev_alloc(&L.grads, 4ull * MLP_NPARAM));
  CU(dev_alloc(&L.adam_m, 4ull * MLP_NPARAM));
  CU(dev_alloc(&L.adam_v, 4ull * MLP_NPARAM));
  CU(dev_alloc(&L.train_img, MLP_IMG_BYTES));
  CU(dev_alloc(&L.bias, 4ull * MLP_BIAS_WORDS));
  CU(dev_alloc(&L.tc_img, mlp_tc_image_bytes()));
  return FDF_SUCCESS;
}

int ensure_scratch(FdfContext *ctx, int B) {
  LocatorState &L = ctx->loc;
  if (L.batch_cap >= B && L.scratch) return FDF_SUCCESS;
  cfree(L.scratch);
  L.batch_cap = 0;
  CU(dev_alloc(&L.scratch, scratch_bytes(B)));
  L.batch_cap = B;
  return FDF_SUCCESS;
}

void set_norm(FdfContext *ctx) {
  LocatorState &L = ctx->loc;
  for (int d = 0; d < 3; ++d) {
    const double lo = ctx->bbox_h[d], hi = ctx->bbox_h[3 + d];
    L.norm.centre[d] = (float)(0.5 * (lo + hi));
    L.norm.inv_half[d] = (float)(2.0 / (hi - lo));
  }
}

// The weights' images: bfloat16 for training, the inference kernel's operand type and biases.
void refresh_weights(FdfContext *ctx, cudaStream_t s) {
  LocatorState &L = ctx->loc;
  mlp_pack_tc(L.params, L.train_img, 1, s);
  mlp_pack_bias(L.params, L.bias, s);
  mlp_pack_tc(L.params, L.tc_img, L.infer_bf16, s);
  ctx->launches += 3;
}

// Output scale of the loss: errors are measured in cells per axis.
void loss_scale(const FdfContext *ctx, float sc[3]) {
  const int N[3] = {ctx->g.IM, ctx->g.JM, ctx->g.KM};
  for (int d = 0; d < 3; ++d) sc[d] = 0.5f * (float)N[d];
}

}  // namespace

void locator_free(FdfContext *ctx) {
  LocatorState &L = ctx->loc;
  cfree(L.params); cfree(L.grads); cfree(L.adam_m); cfree(L.adam_v); cfree(L.train_img);
  cfree(L.bias); cfree(L.tc_img); cfree(L.pending); cfree(L.guess); cfree(L.scratch); cfree(L.pflag);
  cfree(L.scan_sums);
  L.pending_cap = 0;
  L.batch_cap = 0;
  L.has_params = false;
}

int locator_reserve(FdfContext *ctx) {
  LocatorState &L = ctx->loc;
  if (L.pending_cap >= ctx->cap && L.pending) return FDF_SUCCESS;
  cfree(L.pending); cfree(L.guess); cfree(L.pflag); cfree(L.scan_sums);
  L.pending_cap = 0;
  CU(dev_alloc(&L.pending, 4ull * ctx->cap));
  CU(dev_alloc(&L.guess, 4ull * ctx->cap));
  CU(dev_alloc(&L.pflag, 4ull * (2 * ((ctx->cap + 31) / 32) + 1)));
  CU(dev_alloc(&L.scan_sums, 4ull * scan_scratch_words(ctx->cap + 1)));
  L.pending_cap = ctx->cap;
  return FDF_SUCCESS;
}

extern "C" {

int fdf_LocatorInit(FdfContext *ctx, uint64_t seed) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorInit: call fdf_SetGrid first");
  CU(cudaSetDevice(ctx->device));
  int r = alloc_params(ctx);
  if (r) return r;
  std::vector<float> p(MLP_NPARAM);
  mlp_init_params_host(seed, p.data());
  LocatorState &L = ctx->loc;
  set_norm(ctx);
  CU(cudaMemcpyAsync(L.params, p.data(), 4ull * MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemsetAsync(L.adam_m, 0, 4ull * MLP_NPARAM, ctx->stream));
  CU(cudaMemsetAsync(L.adam_v, 0, 4ull * MLP_NPARAM, ctx->stream));
  L.adam_t = 0;
  refresh_weights(ctx, ctx->stream);
  CHECK_LAUNCH();
  CU(cudaStreamSynchronize(ctx->stream));
  L.has_params = true;
  return FDF_SUCCESS;
}

int fdf_LocatorSetParams(FdfContext *ctx, const float *params, int64_t n) {
  if (!ctx || !params) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatorSetParams: null argument");
  if (n != MLP_NPARAM) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorSetParams: expected FDF_LOCATOR_NPARAM");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorSetParams: call fdf_SetGrid first");
  CU(cudaSetDevice(ctx->device));
  int r = alloc_params(ctx);
  if (r) return r;
  LocatorState &L = ctx->loc;
  set_norm(ctx);
  CU(cudaMemcpyAsync(L.params, params, 4ull * MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemsetAsync(L.adam_m, 0, 4ull * MLP_NPARAM, ctx->stream));
  CU(cudaMemsetAsync(L.adam_v, 0, 4ull * MLP_NPARAM, ctx->stream));
  L.adam_t = 0;
  refresh_weights(ctx, ctx->stream);
  CHECK_LAUNCH();
  CU(cudaStreamSynchronize(ctx->stream));
  L.has_params = true;
  return FDF_SUCCESS;
}

int fdf_LocatorGetParams(FdfContext *ctx, float *params, int64_t n) {
  if (!ctx || !params) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatorGetParams: null argument");
  if (n != MLP_NPARAM) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorGetParams: expected FDF_LOCATOR_NPARAM");
  if (!ctx->loc.has_params) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorGetParams: no locator");
  CU(cudaSetDevice(ctx->device));
  CU(cudaMemcpyAsync(params, ctx->loc.params, 4ull * MLP_NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

int fdf_LocatorGetNormalization(FdfContext *ctx, float *centre, float *inv_half) {
  if (!ctx || !centre || !inv_half) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatorGetNormalization: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorGetNormalization: no grid");
  set_norm(ctx);
  for (int d = 0; d < 3; ++d) { centre[d] = ctx->loc.norm.centre[d]; inv_half[d] = ctx->loc.norm.inv_half[d]; }
  return FDF_SUCCESS;
}

// fdf_LocatorGradients, and with stall_test the time-out test of fdf_TestLocatorTrainTimeout
// (the training kernel alone, no MMA issued; grads and loss unused).
static int locator_gradients(FdfContext *ctx, const float *xhat, const float *target, int64_t batch, float *grads,
                             float *loss, int stall_test) {
  if (!ctx || !xhat || !target || (!stall_test && (!grads || !loss)))
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatorGradients: null argument");
  if (batch < 1 || batch > 65536) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorGradients: batch in [1, 65536]");
  if (!ctx->loc.has_params) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorGradients: no locator");
  CU(cudaSetDevice(ctx->device));
  const int B = (int)batch;
  int r = ensure_scratch(ctx, B);
  if (r) return r;
  TrainScratch S = carve_scratch(ctx->loc.scratch, ctx->loc.batch_cap);
  cudaStream_t s = ctx->stream;
  LocatorState &L = ctx->loc;
  CU(cudaMemcpyAsync(S.xs, xhat, 12ull * B, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(S.ts, target, 12ull * B, cudaMemcpyHostToDevice, s));
  CU(cudaMemsetAsync(S.err, 0, 4, s));
  float sc[3];
  loss_scale(ctx, sc);
  float *d_loss = S.loss_part + mlp_train_tiles(B);
  CU(cudaMemsetAsync(d_loss, 0, 4, s));
  mlp_pack_tc(L.params, L.train_img, 1, s);
  mlp_train_step(L.train_img, L.params, S.xs, S.ts, B, 0, 0, 0, B, sc, S.part, S.loss_part, S.err, s, stall_test);
  ctx->launches += 2;
  if (!stall_test) {
    mlp_train_update(S.part, mlp_train_tiles(B), S.loss_part, L.params, L.grads, nullptr, nullptr, L.train_img,
                     d_loss, 0, 0.f, 1.f, 1.f, s);
    ctx->launches += 1;
  }
  CHECK_LAUNCH();
  unsigned int errw = 0;
  if (!stall_test) {
    CU(cudaMemcpyAsync(grads, ctx->loc.grads, 4ull * MLP_NPARAM, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(loss, d_loss, 4, cudaMemcpyDeviceToHost, s));
  }
  CU(cudaMemcpyAsync(&errw, S.err, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if (errw & ERRBIT_TC_TIMEOUT) return fail(ctx, FDF_ERR_GPU, "fdf_LocatorGradients: tensor-core wait timed out");
  return FDF_SUCCESS;
}

int fdf_LocatorGradients(FdfContext *ctx, const float *xhat, const float *target, int64_t batch, float *grads,
                         float *loss) {
  return locator_gradients(ctx, xhat, target, batch, grads, loss, 0);
}

int fdf_TestLocatorTrainTimeout(FdfContext *ctx, const float *xhat, const float *target, int64_t batch) {
  return locator_gradients(ctx, xhat, target, batch, nullptr, nullptr, 1);
}

int fdf_LocatorTrain(FdfContext *ctx, int64_t n_samples, uint64_t seed, int64_t steps, int64_t batch, double lr,
                     float *loss_history) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorTrain: call fdf_SetGrid first");
  if (n_samples < 1 || n_samples > 0x7fffffffLL || steps < 0 || batch < 16 || batch > 65536 || !(lr > 0.0))
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorTrain: argument out of range");
  CU(cudaSetDevice(ctx->device));
  if (!ctx->loc.has_params) {
    int r = fdf_LocatorInit(ctx, seed);
    if (r) return r;
  }
  LocatorState &L = ctx->loc;
  set_norm(ctx);
  cudaStream_t s = ctx->stream;
  const GridDims &g = ctx->g;
  const long long n = n_samples;
  // --- location pairs from the walking search
  void *tmp_swarm = nullptr;
  CU(cudaMalloc(&tmp_swarm, swarm_bytes_per_buf((int)n)));
  SwarmBuf tb;
  carve_swarm((char *)tmp_swarm, (int)n, tb);
  DevCounters *tc = nullptr;
  unsigned int *keys = nullptr, *hist = nullptr, *flag = nullptr, *slot = nullptr, *sums = nullptr;
  float *xs = nullptr, *ts = nullptr, *hist_loss = nullptr;
  auto release = [&]() {
    cudaStreamSynchronize(s);
    cudaFree(tmp_swarm); cudaFree(tc); cudaFree(keys); cudaFree(hist); cudaFree(flag); cudaFree(slot);
    cudaFree(sums); cudaFree(xs); cudaFree(ts); cudaFree(hist_loss);
  };
#define CUT(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      release();                                                                     \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? FDF_ERR_MEM : FDF_ERR_GPU,  \
                  std::string(#call) + ": " + cudaGetErrorString(e_));               \
    }                                                                                \
  } while (0)
  CUT(cudaMalloc((void **)&tc, sizeof(DevCounters)));
  CUT(cudaMalloc((void **)&keys, 4ull * n));
  CUT(cudaMalloc((void **)&hist, 4ull * (g.Nc + 2)));
  CUT(cudaMalloc((void **)&flag, 4ull * n));
  CUT(cudaMalloc((void **)&slot, 4ull * n));
  CUT(cudaMalloc((void **)&sums, 4ull * scan_scratch_words(n)));
  DevCounters c0{};
  c0.n = (int)n;
  c0.n_sorted = (int)n;
  CUT(cudaMemcpyAsync(tc, &c0, sizeof(c0), cudaMemcpyHostToDevice, s));
  CUT(cudaMemsetAsync(hist, 0, 4ull * (g.Nc + 2), s));
  launch_seed(ctx->coor, g, n, seed, 0, 1, 0, 0.0, tb, s);
  launch_locate(tb, (int)n, g, ctx->table32, ctx->planes, 0.0, 0, ctx->bbox, 0, tc, keys, nullptr, hist,
                  ctx->sentinel, s);
  mlp_flag_located(tb.cell, tb.status, n, flag, s);
  CUT(cudaMemcpyAsync(slot, flag, 4ull * n, cudaMemcpyDeviceToDevice, s));
  exclusive_scan_u32(slot, n, sums, s);
  CUT(cudaGetLastError());
  unsigned int last[2] = {0, 0};
  CUT(cudaMemcpyAsync(&last[0], slot + n - 1, 4, cudaMemcpyDeviceToHost, s));
  CUT(cudaMemcpyAsync(&last[1], flag + n - 1, 4, cudaMemcpyDeviceToHost, s));
  unsigned int err = 0;
  CUT(cudaMemcpyAsync(&err, &tc->err, 4, cudaMemcpyDeviceToHost, s));
  CUT(cudaStreamSynchronize(s));
  if (err & ERRBIT_DEGENERATE) {
    release();
    return fail(ctx, FDF_ERR_USER, "Degenerate plane detected (normal vector is near zero).");
  }
  const long long m = (long long)last[0] + last[1];
  if (m == 0) {
    release();
    return fail(ctx, FDF_ERR_ARG_WRONG, "fdf_LocatorTrain: the walk located none of the sample points");
  }
  CUT(cudaMalloc((void **)&xs, 12ull * m));
  CUT(cudaMalloc((void **)&ts, 12ull * m));
  mlp_make_samples(tb.x, tb.y, tb.z, tb.cell, slot, flag, n, L.norm, g, xs, ts, s);
  ctx->launches += 4 + 3;
  // --- training
  const int B = (int)batch;
  int r = ensure_scratch(ctx, B);
  if (r) { release(); return r; }
  TrainScratch S = carve_scratch(L.scratch, L.batch_cap);
  CUT(cudaMalloc((void **)&hist_loss, 4ull * (steps > 0 ? steps : 1)));
  CUT(cudaMemsetAsync(S.err, 0, 4, s));
  float sc[3];
  loss_scale(ctx, sc);
  const int tiles = mlp_train_tiles(B);
  mlp_pack_tc(L.params, L.train_img, 1, s);
  ctx->launches += 1;
  const double pi = 3.14159265358979323846;
  for (long long t = 0; t < steps; ++t) {
    mlp_train_step(L.train_img, L.params, xs, ts, m, seed ^ 0x5DEECE66DULL, t, 1, B, sc, S.part, S.loss_part, S.err,
                   s);
    const double lr_t = lr * (0.02 + 0.98 * 0.5 * (1.0 + std::cos(pi * (double)t / (double)steps)));
    L.adam_t += 1;
    const double c1 = 1.0 - std::pow(0.9, (double)L.adam_t), c2 = 1.0 - std::pow(0.999, (double)L.adam_t);
    mlp_train_update(S.part, tiles, S.loss_part, L.params, L.grads, L.adam_m, L.adam_v, L.train_img, hist_loss + t, 1,
                     (float)lr_t, (float)c1, (float)c2, s);
    ctx->launches += 2;
    if ((t & 255) == 255) CUT(cudaGetLastError());
  }
  refresh_weights(ctx, s);
  CUT(cudaGetLastError());
  if (loss_history && steps > 0)
    CUT(cudaMemcpyAsync(loss_history, hist_loss, 4ull * steps, cudaMemcpyDeviceToHost, s));
  unsigned int errw = 0;
  CUT(cudaMemcpyAsync(&errw, S.err, 4, cudaMemcpyDeviceToHost, s));
  CUT(cudaStreamSynchronize(s));
#undef CUT
  release();
  L.has_params = !(errw & ERRBIT_TC_TIMEOUT);   // weights from a step that timed out are not kept as valid
  if (errw & ERRBIT_TC_TIMEOUT) return fail(ctx, FDF_ERR_GPU, "fdf_LocatorTrain: tensor-core wait timed out");
  return FDF_SUCCESS;
}

// fdf_LocatorPredict, and with stall_test the time-out test of fdf_TestLocatorWaitTimeout.
// The call reports only its own launch's tensor-core time-out (a word of its own, cleared first).
static int locator_predict(FdfContext *ctx, const double *position, int64_t n, int64_t *cell_id, float *outputs,
                           int stall_test) {
  if (!ctx || (n > 0 && (!position || !cell_id))) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatorPredict: null argument");
  if (n < 0 || n > 0x7fffffffLL) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorPredict: n out of range");
  if (!ctx->loc.has_params) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatorPredict: no locator");
  if (n == 0) return FDF_SUCCESS;
  CU(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  std::vector<double> soa(3 * (size_t)n);
  for (int64_t p = 0; p < n; ++p)
    for (int d = 0; d < 3; ++d) soa[d * (size_t)n + p] = position[3 * p + d];
  // one buffer: positions [3][n] f64, outputs [n][3] f32, guesses [n] i32, the error word
  const size_t off_out = 24ull * n, off_guess = off_out + (12ull * n + 255) / 256 * 256,
               off_err = off_guess + (4ull * n + 255) / 256 * 256;
  char *mem = nullptr;
  CU(cudaMalloc((void **)&mem, off_err + 256));
  double *d_pos = (double *)mem;
  float *d_out = (float *)(mem + off_out);
  int *d_guess = (int *)(mem + off_guess);
  unsigned int *d_err = (unsigned int *)(mem + off_err);
  cudaError_t e = cudaMemcpyAsync(d_pos, soa.data(), 24ull * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    mlp_guess_tc(ctx->loc.tc_img, ctx->loc.infer_bf16, ctx->loc.bias, ctx->loc.norm, d_pos, d_pos + n,
                 d_pos + 2 * n, 0, nullptr, nullptr, (int)n, (int)n, ctx->g, d_guess, ctx->num_sms, d_err, s, d_out,
                 stall_test);
    ctx->launches += 1;
    e = cudaGetLastError();
  }
  std::vector<int> gh((size_t)n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gh.data(), d_guess, 4ull * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && outputs) e = cudaMemcpyAsync(outputs, d_out, 12ull * n, cudaMemcpyDeviceToHost, s);
  unsigned int errw = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&errw, d_err, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(mem);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_LocatorPredict: ") + cudaGetErrorString(e));
  if (errw & ERRBIT_TC_TIMEOUT) return fail(ctx, FDF_ERR_GPU, "fdf_LocatorPredict: tensor-core wait timed out");
  const long long IM = ctx->g.IM, JM = ctx->g.JM;
  for (int64_t p = 0; p < n; ++p) {
    const long long c = gh[p];
    cell_id[3 * p] = c % IM;
    cell_id[3 * p + 1] = (c / IM) % JM;
    cell_id[3 * p + 2] = c / (IM * JM);
  }
  return FDF_SUCCESS;
}

int fdf_LocatorPredict(FdfContext *ctx, const double *position, int64_t n, int64_t *cell_id, float *outputs) {
  return locator_predict(ctx, position, n, cell_id, outputs, 0);
}

int fdf_TestLocatorWaitTimeout(FdfContext *ctx, const double *position, int64_t n) {
  if (!ctx || !position) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_TestLocatorWaitTimeout: null argument");
  if (n < 1) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_TestLocatorWaitTimeout: n must be positive");
  std::vector<int64_t> cells(3 * (size_t)n);
  return locator_predict(ctx, position, n, cells.data(), nullptr, 1);
}

int fdf_LocatorSetInferenceType(FdfContext *ctx, int type) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (type != FDF_LOCATOR_BF16 && type != FDF_LOCATOR_F16)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorSetInferenceType: FDF_LOCATOR_BF16 or FDF_LOCATOR_F16");
  LocatorState &L = ctx->loc;
  const int bf16 = type == FDF_LOCATOR_BF16 ? 1 : 0;
  if (bf16 == L.infer_bf16) return FDF_SUCCESS;
  CU(cudaSetDevice(ctx->device));
  L.infer_bf16 = bf16;
  ctx->gen++;   // a captured step holds the launch's operand type
  if (L.has_params) {
    mlp_pack_tc(L.params, L.tc_img, L.infer_bf16, ctx->stream);
    ctx->launches += 1;
    CHECK_LAUNCH();
    CU(cudaStreamSynchronize(ctx->stream));
  }
  return FDF_SUCCESS;
}

int fdf_LocatorSetMinDistance(FdfContext *ctx, double cells) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!(cells >= 0.0)) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatorSetMinDistance: cells must be >= 0");
  ctx->loc.far_cells = (float)cells;
  ctx->gen++;   // a captured step holds the value
  return FDF_SUCCESS;
}

int fdf_LocatorGetStats(FdfContext *ctx, int64_t *asked, int64_t *taken, int64_t *guess_evals,
                        int64_t *fallback_evals) {
  // taken: evaluations on the predicted path; guess_evals: evaluations of the walks from P1
  if (!ctx || !asked || !taken || !guess_evals || !fallback_evals) return FDF_ERR_ARG_NULL;
  CU(cudaSetDevice(ctx->device));
  DevCounters c{};
  CU(cudaMemcpyAsync(&c, ctx->cnt, DEVCOUNTERS_HEAD, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  *asked = (int64_t)c.guess_asked_total;
  *taken = (int64_t)c.guess_taken_total;
  *guess_evals = (int64_t)c.guess_evals_total;
  *fallback_evals = (int64_t)c.fallback_evals_total;
  return FDF_SUCCESS;
}

}  // extern "C"
