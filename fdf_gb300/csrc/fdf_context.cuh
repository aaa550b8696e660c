// fdf_context.cuh -- the device context behind the opaque FdfContext of the C ABI,
// shared by the API translation units (fdf_api.cu, fdf_locator.cu).
#pragma once
#include "fdf_internal.cuh"
#include "fdf_mlp.cuh"
#include "../../include/fdf_gb300.h"

#include <string>
#include <utility>
#include <vector>

// The learned start-cell locator of one context (FDF_FORM_LEARNED_FP32).
struct LocatorState {
  bool has_params = false;
  float *params = nullptr;            // [MLP_NPARAM] FP32 master weights
  float *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  unsigned char *train_img = nullptr; // bfloat16 image of the weights the training step reads
  unsigned char *tc_img = nullptr;    // inference weights as the tcgen05 kernel's shared-memory image
  int infer_bf16 = 1;                 // inference operands: bfloat16 (1) or half precision (0)
  float *bias = nullptr;
  MlpNorm norm{};
  long long adam_t = 0;
  float far_cells = 2.0f;             // particles at least this far past their cell get a guess
  // per-particle buffers of the learned form's locate
  unsigned int *pending = nullptr;    // [cap]: slots that left their previous cell, in slot order
  unsigned int *pflag = nullptr;      // [2W+1], W = ceil(cap/32): per warp of slots a mask, then the
                                      // counts' exclusive scan
  unsigned int *scan_sums = nullptr;
  int *guess = nullptr;               // [cap]: learned start cell of pending[t]
  int pending_cap = 0;
  // training scratch for batches up to `batch_cap`
  int batch_cap = 0;
  void *scratch = nullptr;
};

struct FdfContext {
  int device = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t ev_scan = nullptr, ev_corner = nullptr, ev_xfer = nullptr;
  GridDims g{};
  bool has_grid = false, has_ucat = false;
  double *coor = nullptr, *planes = nullptr, *ucat = nullptr, *corner = nullptr, *bbox = nullptr;
  double *count = nullptr, *avg = nullptr, *fi = nullptr, *fj = nullptr, *fk = nullptr;
  // precision form (FDF_FORM_FP32)
  int form = FDF_FORM_PLAIN_FP64;
  float *table32 = nullptr, *ucat32 = nullptr, *corner32 = nullptr, *fbox = nullptr;
  float *count32 = nullptr, *avg32 = nullptr, *fi32 = nullptr, *fj32 = nullptr, *fk32 = nullptr;
  double bbox_h[6] = {0, 0, 0, 0, 0, 0};
  // momentum face deposit (fdf_SetMomentumDeposit): SoA [3][faces] per face family
  bool momentum = false;
  double *mom = nullptr;   // mi | mj | mk, 3 (nfi + nfj + nfk) doubles
  float *mom32 = nullptr;
  double dt = 0.0, volume = 1.0;
  int cap = 0;
  SwarmBuf buf[2];
  int cur = 0;
  void *swarm_mem = nullptr;
  unsigned int *keys = nullptr, *perm = nullptr;   // [cap]: cell key per slot, sorted slot -> previous slot
  unsigned int *rank = nullptr;                    // [cap]: rank of the slot's particle within its new cell
  unsigned int *cell_start = nullptr;              // [Nc+2]: histogram, then its exclusive scan
  unsigned int *scan_sums = nullptr;
  DevCounters *cnt = nullptr;
  void *staging = nullptr;
  size_t staging_bytes = 0;
  int xfer_route = FDF_TRANSFER_AUTO;     // fdf_SetTransferRoute
  int route_up = -1, route_down = -1;     // AUTO: the route measured faster per direction (-1: not yet)
  unsigned int sentinel = 0;
  bool swarm_set = false;
  bool layout_ok = false;   // the held particles are sorted by cell and cell_start matches them
  int swarm_form = FDF_FORM_PLAIN_FP64;   // form the swarm's device arrays are held in
  int out_form = FDF_FORM_PLAIN_FP64;     // form of the last deposits
  bool out_momentum = false;              // the last deposits include the momentum
  long long launches = 0;
  // stage timing: events recorded on the context stream between pipeline stages
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, std::pair<size_t, size_t>>> ev_spans;   // (stage, (start ev, end ev))
  std::string last_error;
  int num_sms = 0;
  LocatorState loc;
  // Eulerian input (fdf_eulerian.cu): face velocity and the per-cell Contra2Cart table
  double *ucont = nullptr;       // [Nn][3] node-sized, as the reference's lUcont
  double *c2c_table = nullptr;   // [10][Nc], built on the first fdf_Contra2Cart of a grid
  int c2c_rc = FDF_SUCCESS;      // the table build's error (a near-zero determinant)
  std::string c2c_msg;
  int c2c_flipped = 0;
  bool c2c_half = false;         // every tabled value mid-range: the halved Contra2Cart applies
  // fdf_AdvanceSteps replays one captured step per swarm buffer parity; `gen` counts the
  // changes of anything a captured step bakes in (pointers, kernel arguments, form)
  long long gen = 1;
  cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
  long long graph_gen[2] = {0, 0};
  long long eager_gen = 0;   // generation of the last eager step
};


// forms whose swarm is held in the precision-form arrays
inline bool form_is32(int form) { return form == FDF_FORM_FP32 || form == FDF_FORM_LEARNED_FP32; }

// Stage ids reported by fdf_GetStageTimes.
enum { FDF_STAGE_CORNER = 0, FDF_STAGE_LOCATE = 1, FDF_STAGE_SORT = 2, FDF_STAGE_WAIT = 3,
       FDF_STAGE_GATHER_INTERP = 4, FDF_STAGE_DEPOSIT = 5, FDF_STAGE_GUESS = 6, FDF_STAGE_GUESS_WALK = 7,
       FDF_STAGE_CONTRA2CART = 8, FDF_NUM_STAGES = 9 };

// Records a pooled timing event on `stream`; returns its index in ctx->ev_pool.
inline size_t record_event(FdfContext *ctx, cudaStream_t stream) {
  if (ctx->ev_used == ctx->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return (size_t)-1;
    ctx->ev_pool.push_back(e);
  }
  size_t id = ctx->ev_used++;
  cudaEventRecord(ctx->ev_pool[id], stream);
  return id;
}

// Frees the Eulerian-input buffers (face velocity, Contra2Cart table) of the context's grid.
void eulerian_free(FdfContext *ctx);

inline int fail(FdfContext *ctx, int code, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

#define CU(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? FDF_ERR_MEM : FDF_ERR_GPU,       \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

#define CHECK_LAUNCH()                                                                    \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("launch: ") + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
inline void cfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

// Device allocations of the context's long-lived buffers go through dev_alloc, so that a test
// can make them fail on the host (fdf_TestFailDeviceAllocations) and check that the context
// is left refusing work instead of holding freed pointers.
cudaError_t dev_alloc_hooked(void **p, size_t bytes);
template <typename T>
inline cudaError_t dev_alloc(T **p, size_t bytes) {
  return dev_alloc_hooked(reinterpret_cast<void **>(p), bytes);
}


// Bytes of one swarm buffer, a multiple of 256: the second buffer of the pair starts at this
// offset, and its arrays keep the 256-B alignment of the first's (the deposit's bulk copies need
// 16-B aligned sources).
inline size_t swarm_bytes_per_buf(int cap) {
  const size_t b =
      (size_t)cap * (10 * sizeof(double) + 7 * sizeof(float) + sizeof(long long) + sizeof(int) + 1) + 24 * 256;
  return (b + 255) / 256 * 256;
}

inline void carve_swarm(char *p, int cap, SwarmBuf &b) {
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) / 256 * 256;
    return r;
  };
  b.x = (double *)take(8ull * cap); b.y = (double *)take(8ull * cap); b.z = (double *)take(8ull * cap);
  b.u = (double *)take(8ull * cap); b.v = (double *)take(8ull * cap); b.w = (double *)take(8ull * cap);
  b.a1 = (double *)take(8ull * cap); b.a2 = (double *)take(8ull * cap); b.a3 = (double *)take(8ull * cap);
  b.P = (double *)take(8ull * cap);
  b.uf = (float *)take(4ull * cap); b.vf = (float *)take(4ull * cap); b.wf = (float *)take(4ull * cap);
  b.a1f = (float *)take(4ull * cap); b.a2f = (float *)take(4ull * cap); b.a3f = (float *)take(4ull * cap);
  b.Pf = (float *)take(4ull * cap);
  b.pid = (long long *)take(8ull * cap);
  b.cell = (int *)take(4ull * cap);
  b.status = (unsigned char *)take((size_t)cap);
}


// fdf_locator.cu
void locator_free(FdfContext *ctx);
// Learned form: make sure the per-particle guess buffers hold ctx->cap particles.
int locator_reserve(FdfContext *ctx);
