// fdf_api.cu -- the C ABI (include/fdf_gb300.h): device context, transfers, and
// the step pipeline on the context's stream.
//
// Step pipeline (no host round trip):
//   locate  (advect, walk from the previous cell, weights; histogram of the new cells;
//            removed particles get key Nc and no slot)
//   scan of the histogram -> cell_start[Nc+2]
//   [side stream] center->corner for nodes next to occupied cells (FP64-bound, runs
//                 concurrently with the integer-bound slot assignment)
//   slot assignment (counting sort) + per-cell ordering by PID
//   gather + interpolate into the alternate buffer (sorted order)
//   deposit (cell count / P average, face volumes) from the sorted segments
#include "fdf_context.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <atomic>

namespace {

// Allocations left before dev_alloc starts failing (fdf_TestFailDeviceAllocations); -1: no limit.
std::atomic<long long> g_alloc_budget{-1};

}  // namespace

cudaError_t dev_alloc_hooked(void **p, size_t bytes) {
  long long b = g_alloc_budget.load();
  while (b >= 0) {
    if (b == 0) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
    if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
  }
  return cudaMalloc(p, bytes);
}

extern "C" {

int fdf_TestFailDeviceAllocations(int64_t after) {
  g_alloc_budget.store(after < 0 ? -1 : (long long)after);
  return FDF_SUCCESS;
}

int fdf_ContextCreate(FdfContext **out, int device) {
  FdfContext *ctx = nullptr;
  if (!out) return FDF_ERR_ARG_NULL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FDF_ERR_GPU;
  if (device < 0 || device >= ndev) return FDF_ERR_ARG_OUTOFRANGE;
  ctx = new FdfContext();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_scan, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_corner, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_xfer, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->cnt, sizeof(DevCounters));
  if (e == cudaSuccess) e = cudaMemset(ctx->cnt, 0, sizeof(DevCounters));
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->bbox, 6 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->fbox, 16 * sizeof(float));
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    fdf_ContextDestroy(ctx);
    return FDF_ERR_GPU;
  }
  *out = ctx;
  return FDF_SUCCESS;
}

int fdf_ContextDestroy(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cfree(ctx->coor); cfree(ctx->planes); cfree(ctx->ucat); cfree(ctx->corner); cfree(ctx->bbox);
  cfree(ctx->count); cfree(ctx->avg); cfree(ctx->fi); cfree(ctx->fj); cfree(ctx->fk);
  cfree(ctx->table32); cfree(ctx->ucat32); cfree(ctx->corner32); cfree(ctx->count32); cfree(ctx->avg32);
  cfree(ctx->fi32); cfree(ctx->fj32); cfree(ctx->fk32); cfree(ctx->fbox); cfree(ctx->mom); cfree(ctx->mom32);
  eulerian_free(ctx);
  if (ctx->side) cudaStreamSynchronize(ctx->side);
  cfree(ctx->swarm_mem); cfree(ctx->keys); cfree(ctx->perm); cfree(ctx->rank);
  cfree(ctx->cell_start); cfree(ctx->scan_sums); cfree(ctx->cnt); cfree(ctx->staging);
  locator_free(ctx);
  for (auto &gx : ctx->step_graph)
    if (gx) cudaGraphExecDestroy(gx);
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->ev_scan) cudaEventDestroy(ctx->ev_scan);
  if (ctx->ev_corner) cudaEventDestroy(ctx->ev_corner);
  if (ctx->ev_xfer) cudaEventDestroy(ctx->ev_xfer);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FDF_SUCCESS;
}

int fdf_SetGrid(FdfContext *ctx, int64_t IM, int64_t JM, int64_t KM, const double *coor) {
  if (!ctx || !coor) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_SetGrid: null argument");
  if (IM <= 0 || JM <= 0 || KM <= 0)   // grid.c:41-44
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SetGrid: grid dimensions (IM, JM, KM) must be positive");
  long long Nc = IM * JM * KM;
  long long Nn = (IM + 1) * (JM + 1) * (KM + 1);
  if (Nc + 2 > scan_max_count() || Nn >= 0x7fffffffLL)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SetGrid: too many cells or nodes (max 134M cells)");
  CU(cudaSetDevice(ctx->device));
  CU(cudaStreamSynchronize(ctx->stream));
  // From here on the old grid is gone: until every buffer of the new one is in place the
  // context refuses work (and the captured step graphs, which hold the old addresses, are
  // invalidated), so a failed allocation below leaves no call able to touch freed memory.
  ctx->has_grid = false;
  ctx->has_ucat = false;
  ctx->swarm_set = false;
  ctx->layout_ok = false;
  ctx->loc.has_params = false;   // a locator is trained for one grid
  ctx->gen++;
  cfree(ctx->coor); cfree(ctx->planes); cfree(ctx->ucat); cfree(ctx->corner);
  cfree(ctx->count); cfree(ctx->avg); cfree(ctx->fi); cfree(ctx->fj); cfree(ctx->fk); cfree(ctx->cell_start);
  cfree(ctx->scan_sums);
  cfree(ctx->table32); cfree(ctx->ucat32); cfree(ctx->corner32); cfree(ctx->count32); cfree(ctx->avg32);
  cfree(ctx->fi32); cfree(ctx->fj32); cfree(ctx->fk32); cfree(ctx->mom); cfree(ctx->mom32);
  eulerian_free(ctx);
  ctx->momentum = false;
  GridDims g{};
  g.IM = (int)IM; g.JM = (int)JM; g.KM = (int)KM; g.Nc = Nc; g.Nn = Nn;
  g.fIM.init((unsigned)IM); g.fJM.init((unsigned)JM); g.fMX.init((unsigned)(IM + 1)); g.fMY.init((unsigned)(JM + 1));
  ctx->g = g;
  long long nfi = (IM + 1) * JM * KM, nfj = IM * (JM + 1) * KM, nfk = IM * JM * (KM + 1);
  CU(dev_alloc((void **)&ctx->coor, 24ull * Nn));
  CU(dev_alloc((void **)&ctx->planes, 8ull * FDF_ROW * Nc));
  CU(dev_alloc((void **)&ctx->ucat, 24ull * Nc));
  CU(dev_alloc((void **)&ctx->corner, 24ull * Nn));
  CU(dev_alloc((void **)&ctx->count, 8ull * Nn));
  CU(dev_alloc((void **)&ctx->avg, 8ull * Nn));
  CU(dev_alloc((void **)&ctx->fi, 8ull * nfi));
  CU(dev_alloc((void **)&ctx->fj, 8ull * nfj));
  CU(dev_alloc((void **)&ctx->fk, 8ull * nfk));
  CU(dev_alloc((void **)&ctx->table32, 4ull * FDF_ROW32 * Nc));
  CU(dev_alloc((void **)&ctx->ucat32, 12ull * Nc));
  CU(dev_alloc((void **)&ctx->corner32, 12ull * Nn));
  CU(dev_alloc((void **)&ctx->count32, 4ull * Nn));
  CU(dev_alloc((void **)&ctx->avg32, 4ull * Nn));
  CU(dev_alloc((void **)&ctx->fi32, 4ull * nfi));
  CU(dev_alloc((void **)&ctx->fj32, 4ull * nfj));
  CU(dev_alloc((void **)&ctx->fk32, 4ull * nfk));
  CU(cudaMemsetAsync(ctx->ucat32, 0, 12ull * Nc, ctx->stream));
  CU(dev_alloc((void **)&ctx->cell_start, 4ull * (Nc + 2)));
  CU(dev_alloc((void **)&ctx->scan_sums, 4ull * scan_scratch_words(Nc + 2)));
  CU(cudaMemsetAsync(ctx->cell_start, 0, 4ull * (Nc + 2), ctx->stream));
  CU(cudaMemsetAsync(ctx->ucat, 0, 24ull * Nc, ctx->stream));
  CU(cudaMemsetAsync(ctx->corner, 0, 24ull * Nn, ctx->stream));
  CU(cudaMemcpyAsync(ctx->coor, coor, 24ull * Nn, cudaMemcpyHostToDevice, ctx->stream));
  unsigned int *err = nullptr;
  launch_build_planes(ctx->coor, g, ctx->planes, err, ctx->stream);
  CHECK_LAUNCH();
  launch_build_table32(ctx->planes, ctx->coor, g, ctx->table32, ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  ctx->launches += 1;
  // ComputeLocalBoundingBox (grid.c:762-883) on one rank: min/max over every node,
  // widened by 1e-6 -- done on the host, which holds the coordinates.
  double bb[6] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308,
                  -1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
  for (long long q = 0; q < Nn; ++q)
    for (int c = 0; c < 3; ++c) {
      double v = coor[3 * q + c];
      if (v < bb[c]) bb[c] = v;
      if (v > bb[3 + c]) bb[3 + c] = v;
    }
  for (int c = 0; c < 3; ++c) { bb[c] = bb[c] - FDF_BBOX_TOL; bb[3 + c] = bb[3 + c] + FDF_BBOX_TOL; }
  memcpy(ctx->bbox_h, bb, sizeof(bb));
  CU(cudaMemcpyAsync(ctx->bbox, bb, sizeof(bb), cudaMemcpyHostToDevice, ctx->stream));
  // the precision form's FP32 "surely inside" box: any (hi, lo) position with hi strictly
  // inside it lies in [bmin, bmax], because |lo| <= 2^-24 |hi| < margin
  float fb[16] = {0};
  for (int c = 0; c < 3; ++c) {
    const double margin = 0x1p-20 * (std::fabs(bb[c]) + std::fabs(bb[3 + c]) + 1.0);
    const double lo = bb[c] + margin, hi = bb[3 + c] - margin;
    float flo = (float)lo, fhi = (float)hi;
    if ((double)flo < lo) flo = std::nextafter(flo, INFINITY);
    if ((double)fhi > hi) fhi = std::nextafter(fhi, -INFINITY);
    fb[c] = flo;
    fb[4 + c] = fhi;
  }
  CU(cudaMemcpyAsync(ctx->fbox, fb, sizeof(fb), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->sentinel = (unsigned int)Nc;
  ctx->has_grid = true;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_SetUcat(FdfContext *ctx, const double *ucat, int node_sized) {
  if (!ctx || !ucat) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_SetUcat: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_SetUcat: call fdf_SetGrid first");
  const GridDims &g = ctx->g;
  // Host-side transpose to the device SoA layout [3][Nc].
  std::vector<double> soa(3 * (size_t)g.Nc);
  const long long mx = node_sized ? g.IM + 1 : g.IM, my = node_sized ? g.JM + 1 : g.JM;
  for (long long k = 0; k < g.KM; ++k)
    for (long long j = 0; j < g.JM; ++j)
      for (long long i = 0; i < g.IM; ++i) {
        long long c = (k * g.JM + j) * g.IM + i;
        const double *v = ucat + 3 * ((k * my + j) * mx + i);
        soa[c] = v[0]; soa[g.Nc + c] = v[1]; soa[2 * g.Nc + c] = v[2];
      }
  CU(cudaSetDevice(ctx->device));
  CU(cudaMemcpyAsync(ctx->ucat, soa.data(), 24ull * g.Nc, cudaMemcpyHostToDevice, ctx->stream));
  launch_f64_to_f32(ctx->ucat, ctx->ucat32, 3 * g.Nc, ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->has_ucat = true;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_SetTransferRoute(FdfContext *ctx, int route) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (route != FDF_TRANSFER_STAGED && route != FDF_TRANSFER_IN_PLACE && route != FDF_TRANSFER_AUTO)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SetTransferRoute: unknown route");
  ctx->xfer_route = route;
  ctx->route_up = ctx->route_down = -1;   // AUTO measures again
  return FDF_SUCCESS;
}

int fdf_GetTransferRoutes(FdfContext *ctx, int *upload, int *download) {
  if (!ctx || !upload || !download) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetTransferRoutes: null argument");
  *upload = ctx->xfer_route == FDF_TRANSFER_AUTO ? ctx->route_up : ctx->xfer_route;
  *download = ctx->xfer_route == FDF_TRANSFER_AUTO ? ctx->route_down : ctx->xfer_route;
  return FDF_SUCCESS;
}

int fdf_SetForm(FdfContext *ctx, int form) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (form != FDF_FORM_PLAIN_FP64 && form != FDF_FORM_FP32 && form != FDF_FORM_LEARNED_FP32)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SetForm: unknown form");
  ctx->form = form;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_SetTimeStep(FdfContext *ctx, double dt) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  ctx->dt = dt;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_SetParticleVolume(FdfContext *ctx, double volume) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  ctx->volume = volume;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_ReserveParticles(FdfContext *ctx, int64_t capacity) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  // The sort's scan of per-tile digit counts handles up to 2^17 tiles of 4096 keys.
  if (capacity < 0 || capacity > FDF_MAX_PARTICLES)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_ReserveParticles: capacity out of range (max 512M)");
  if (capacity <= ctx->cap && ctx->swarm_mem) return FDF_SUCCESS;
  CU(cudaSetDevice(ctx->device));
  CU(cudaStreamSynchronize(ctx->stream));
  // The held swarm goes with its buffers: until the new ones are all in place the context
  // has no swarm and no capacity, and the captured step graphs (old addresses) are invalid.
  ctx->swarm_set = false;
  ctx->layout_ok = false;
  ctx->cap = 0;
  ctx->buf[0] = SwarmBuf{};
  ctx->buf[1] = SwarmBuf{};
  ctx->staging_bytes = 0;
  ctx->gen++;
  cfree(ctx->swarm_mem); cfree(ctx->keys); cfree(ctx->perm); cfree(ctx->rank); cfree(ctx->staging);
  int cap = (int)(capacity < 256 ? 256 : capacity);   // never zero: the sort always has scratch
  size_t per = swarm_bytes_per_buf(cap);
  CU(dev_alloc(&ctx->swarm_mem, 2 * per));
  CU(dev_alloc(&ctx->keys, 4ull * cap));
  CU(dev_alloc(&ctx->perm, 4ull * cap));
  CU(dev_alloc(&ctx->rank, 4ull * cap));
  CU(dev_alloc(&ctx->staging, (size_t)cap * 120 + 1024));
  carve_swarm((char *)ctx->swarm_mem, cap, ctx->buf[0]);
  carve_swarm((char *)ctx->swarm_mem + per, cap, ctx->buf[1]);
  ctx->staging_bytes = (size_t)cap * 120 + 1024;
  ctx->cap = cap;
  ctx->gen++;
  return FDF_SUCCESS;
}

// The device addresses of the caller's seven DMSwarm arrays when every one is page-locked host
// memory (cudaHostAlloc / cudaHostRegister) and 16-byte aligned, so that the layout kernels can
// read or write them over the host link; false otherwise.
static bool host_views(const void *const a[7], void *v[7]) {
  for (int q = 0; q < 7; ++q) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, a[q]) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || (reinterpret_cast<uintptr_t>(at.devicePointer) & 15u))
      return false;
    v[q] = at.devicePointer;
  }
  return true;
}

// The swarm buffers from particle `off` on.
static SwarmBuf shifted(const SwarmBuf &b, long long off) {
  SwarmBuf r = b;
  auto sh = [off](auto *&p) { if (p) p += off; };
  sh(r.x); sh(r.y); sh(r.z); sh(r.u); sh(r.v); sh(r.w); sh(r.a1); sh(r.a2); sh(r.a3); sh(r.P);
  sh(r.uf); sh(r.vf); sh(r.wf); sh(r.a1f); sh(r.a2f); sh(r.a3f); sh(r.Pf); sh(r.pid); sh(r.cell); sh(r.status);
  return r;
}

// Host <-> device swarm transfers: page-locked arrays are read or written in place by the
// layout kernels (coalesced 16-byte accesses over the host link, no copy calls); other arrays
// go in chunks of particles on two streams, the copies of one chunk (side stream) overlapping
// the layout conversion of the previous one (context stream).
#ifndef FDF_XFER_CHUNKS
#define FDF_XFER_CHUNKS 8
#endif
static int64_t transfer_chunk(int64_t n) {
  return std::max<int64_t>(int64_t(1) << 22, (n + FDF_XFER_CHUNKS - 1) / FDF_XFER_CHUNKS);
}

// The AUTO route's measurement: a warm-up of XFER_WARM particles by each route, then a slice of
// xfer_slice(n) particles by each, timed with events; the rest of the call and later calls of
// that direction take the faster.  Offsets stay multiples of XFER_WARM, so the in-place kernels'
// 16-byte accesses stay aligned.  Calls of fewer than 4 XFER_SLICE_MIN particles are not timed.
constexpr int64_t XFER_WARM = 2048, XFER_SLICE_MIN = int64_t(1) << 20, XFER_SLICE_MAX = int64_t(1) << 22;
static int64_t xfer_slice(int64_t n) {
  if (n < 4 * XFER_SLICE_MIN) return 0;
  return std::min(XFER_SLICE_MAX, n / 4) / XFER_WARM * XFER_WARM;
}

// Times two ranges of one transfer direction: run(0, o, m) by the staged route, run(1, o, m) in
// place; returns the faster route (FDF_TRANSFER_*) and leaves `done` particles transferred.
extern "C++" {
namespace {
template <typename Run>
int calibrate_route(FdfContext *ctx, int64_t m, Run run, int64_t &done, cudaError_t &err) {
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int best = FDF_TRANSFER_STAGED;
  for (auto &e : ev)
    if (err == cudaSuccess) err = cudaEventCreate(&e);
  if (err == cudaSuccess) err = run(0, 0, XFER_WARM);
  if (err == cudaSuccess) err = run(1, XFER_WARM, XFER_WARM);
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->side);
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  const int64_t o = 2 * XFER_WARM;
  if (err == cudaSuccess) err = cudaEventRecord(ev[0], ctx->stream);
  if (err == cudaSuccess) err = run(0, o, m);
  if (err == cudaSuccess) err = cudaEventRecord(ev[1], ctx->side);    // the staged route ends on either
  if (err == cudaSuccess) err = cudaEventRecord(ev[2], ctx->stream);   // stream: time to the later one
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->side);
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  float t_staged = 0.f, t_a = 0.f, t_in = 0.f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&t_staged, ev[0], ev[1]);
  if (err == cudaSuccess) err = cudaEventElapsedTime(&t_a, ev[0], ev[2]);
  t_staged = std::max(t_staged, t_a);
  if (err == cudaSuccess) err = cudaEventRecord(ev[0], ctx->stream);
  if (err == cudaSuccess) err = run(1, o + m, m);
  if (err == cudaSuccess) err = cudaEventRecord(ev[3], ctx->stream);
  if (err == cudaSuccess) err = cudaEventSynchronize(ev[3]);
  if (err == cudaSuccess) err = cudaEventElapsedTime(&t_in, ev[0], ev[3]);
  if (err == cudaSuccess && t_in < t_staged) best = FDF_TRANSFER_IN_PLACE;
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  done = o + 2 * m;
  return best;
}
}  // namespace
}  // extern "C++"

int fdf_SetSwarm(FdfContext *ctx, int64_t n, const double *position, const double *velocity, const double *weight,
                 const double *P, const int64_t *cell_id, const int64_t *pid, const int64_t *status) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (n > 0 && (!position || !velocity || !weight || !P || !cell_id || !pid || !status))
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_SetSwarm: null field pointer");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_SetSwarm: call fdf_SetGrid first");
  if (n < 0) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SetSwarm: negative particle count");
  if (n > ctx->cap || !ctx->swarm_mem) {
    int r = fdf_ReserveParticles(ctx, n);
    if (r) return r;
  }
  CU(cudaSetDevice(ctx->device));
  char *st = (char *)ctx->staging;
  double *d_pos = (double *)st, *d_vel = d_pos + 3 * n, *d_wgt = d_vel + 3 * n, *d_P = d_wgt + 3 * n;
  long long *d_cell = (long long *)(d_P + n), *d_pid = d_cell + 3 * n, *d_st = d_pid + n;
  const void *arrays[7] = {position, velocity, weight, P, cell_id, pid, status};
  void *views[7];
  const bool f32 = form_is32(ctx->form);
  // particles [o, o + m) by the staged (route 0) or the in-place route (1)
  auto run = [&](int route, int64_t o, int64_t m) -> cudaError_t {
    if (m <= 0) return cudaSuccess;
    if (route == 1) {
      const void *v[7];
      const int bs[7] = {3, 3, 3, 1, 3, 1, 1};
      for (int q = 0; q < 7; ++q) v[q] = static_cast<const double *>(views[q]) + bs[q] * o;
      launch_swarm_from_host(v, (int)m, ctx->g, shifted(ctx->buf[0], o), f32, ctx->stream);
      ctx->launches += 1;
      return cudaGetLastError();
    }
    // the side stream starts after everything already queued on the context stream
    cudaError_t e = cudaEventRecord(ctx->ev_xfer, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->side, ctx->ev_xfer, 0);
    const int64_t chunk = transfer_chunk(n);
    for (int64_t c = o; c < o + m && e == cudaSuccess; c += chunk) {
      const int64_t k = std::min(chunk, o + m - c);
      const cudaMemcpyKind h2d = cudaMemcpyHostToDevice;
      e = cudaMemcpyAsync(d_pos + 3 * c, position + 3 * c, 24ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_vel + 3 * c, velocity + 3 * c, 24ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_wgt + 3 * c, weight + 3 * c, 24ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_P + c, P + c, 8ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_cell + 3 * c, cell_id + 3 * c, 24ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_pid + c, pid + c, 8ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d_st + c, status + c, 8ull * k, h2d, ctx->side);
      if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_xfer, ctx->side);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_xfer, 0);
      if (e != cudaSuccess) break;
      const SwarmBuf b = shifted(ctx->buf[0], c);
      if (f32)
        launch_swarm_from_aos32(d_pos + 3 * c, d_vel + 3 * c, d_wgt + 3 * c, d_P + c, d_cell + 3 * c, d_pid + c,
                                d_st + c, (int)k, ctx->g, b, ctx->stream);
      else
        launch_swarm_from_aos(d_pos + 3 * c, d_vel + 3 * c, d_wgt + 3 * c, d_P + c, d_cell + 3 * c, d_pid + c,
                              d_st + c, (int)k, ctx->g, b, ctx->stream);
      ctx->launches += 1;
      e = cudaGetLastError();
    }
    return e;
  };
  ctx->cur = 0;
  if (n > 0) {
    const bool pinned = ctx->xfer_route != FDF_TRANSFER_STAGED && host_views(arrays, views);
    int route = FDF_TRANSFER_STAGED;
    int64_t done = 0;
    cudaError_t e = cudaSuccess;
    if (pinned && ctx->xfer_route == FDF_TRANSFER_IN_PLACE) {
      route = FDF_TRANSFER_IN_PLACE;
    } else if (pinned && ctx->route_up >= 0) {
      route = ctx->route_up;
    } else if (pinned && xfer_slice(n) > 0) {
      route = calibrate_route(ctx, xfer_slice(n), run, done, e);
      if (e == cudaSuccess) ctx->route_up = route;
    }
    if (e == cudaSuccess) e = run(route == FDF_TRANSFER_IN_PLACE ? 1 : 0, done, n - done);
    if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_SetSwarm: ") + cudaGetErrorString(e));
  }
  DevCounters c{};
  c.n = (int)n;
  c.n_sorted = (int)n;
  CU(cudaMemcpyAsync(ctx->cnt, &c, sizeof(c), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->cur = 0;
  ctx->swarm_set = true;
  ctx->layout_ok = false;
  ctx->gen++;
  ctx->swarm_form = ctx->form;
  return FDF_SUCCESS;
}

int fdf_SeedParticles(FdfContext *ctx, int64_t n, uint64_t seed, int start_in_generating_cell, int64_t pid_base,
                      double P) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_SeedParticles: call fdf_SetGrid first");
  if (n < 0) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_SeedParticles: negative particle count");
  if (n > ctx->cap || !ctx->swarm_mem) {
    int r = fdf_ReserveParticles(ctx, n);
    if (r) return r;
  }
  CU(cudaSetDevice(ctx->device));
  ctx->cur = 0;
  launch_seed(ctx->coor, ctx->g, n, seed, pid_base, start_in_generating_cell ? 1 : 0,
              form_is32(ctx->form) ? 1 : 0, P, ctx->buf[0], ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  DevCounters c{};
  c.n = (int)n;
  c.n_sorted = (int)n;
  CU(cudaMemcpyAsync(ctx->cnt, &c, sizeof(c), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->swarm_set = true;
  ctx->layout_ok = false;
  ctx->gen++;
  ctx->swarm_form = ctx->form;
  return FDF_SUCCESS;
}

int fdf_GetSwarmSize(FdfContext *ctx, int64_t *n) {
  if (!ctx || !n) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetSwarmSize: null argument");
  CU(cudaSetDevice(ctx->device));
  int v = 0;
  CU(cudaMemcpyAsync(&v, &ctx->cnt->n_sorted, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  *n = v;
  return FDF_SUCCESS;
}

int fdf_GetSwarm(FdfContext *ctx, int64_t n_max, int64_t *n_out, double *position, double *velocity, double *weight,
                 double *P, int64_t *cell_id, int64_t *pid, int64_t *status) {
  if (!ctx || !n_out) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetSwarm: null argument");
  int64_t n = 0;
  int r = fdf_GetSwarmSize(ctx, &n);
  if (r) return r;
  *n_out = n;
  if (n > n_max) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_GetSwarm: output arrays smaller than the swarm");
  if (n == 0) return FDF_SUCCESS;
  if (!position || !velocity || !weight || !P || !cell_id || !pid || !status)
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetSwarm: null field pointer");
  char *st = (char *)ctx->staging;
  double *d_pos = (double *)st, *d_vel = d_pos + 3 * n, *d_wgt = d_vel + 3 * n, *d_P = d_wgt + 3 * n;
  long long *d_cell = (long long *)(d_P + n), *d_pid = d_cell + 3 * n, *d_st = d_pid + n;
  const void *arrays[7] = {position, velocity, weight, P, cell_id, pid, status};
  void *views[7];
  const bool f32 = form_is32(ctx->swarm_form);
  const SwarmBuf &src = ctx->buf[ctx->cur];
  // particles [o, o + m) by the staged (route 0) or the in-place route (1)
  auto run = [&](int route, int64_t o, int64_t m) -> cudaError_t {
    if (m <= 0) return cudaSuccess;
    if (route == 1) {
      void *v[7];
      const int bs[7] = {3, 3, 3, 1, 3, 1, 1};
      for (int q = 0; q < 7; ++q) v[q] = static_cast<double *>(views[q]) + bs[q] * o;
      launch_swarm_to_host(shifted(src, o), (int)m, ctx->g, v, f32, ctx->stream);
      ctx->launches += 1;
      return cudaGetLastError();
    }
    const int64_t chunk = transfer_chunk(n);
    cudaError_t e = cudaSuccess;
    for (int64_t c = o; c < o + m && e == cudaSuccess; c += chunk) {
      const int64_t k = std::min(chunk, o + m - c);
      const SwarmBuf b = shifted(src, c);
      if (f32)
        launch_swarm_to_aos32(b, (int)k, ctx->g, d_pos + 3 * c, d_vel + 3 * c, d_wgt + 3 * c, d_P + c,
                              d_cell + 3 * c, d_pid + c, d_st + c, ctx->stream);
      else
        launch_swarm_to_aos(b, (int)k, ctx->g, d_pos + 3 * c, d_vel + 3 * c, d_wgt + 3 * c, d_P + c, d_cell + 3 * c,
                            d_pid + c, d_st + c, ctx->stream);
      ctx->launches += 1;
      e = cudaGetLastError();
      const cudaMemcpyKind d2h = cudaMemcpyDeviceToHost;
      if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_xfer, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->side, ctx->ev_xfer, 0);
      if (e == cudaSuccess) e = cudaMemcpyAsync(position + 3 * c, d_pos + 3 * c, 24ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(velocity + 3 * c, d_vel + 3 * c, 24ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(weight + 3 * c, d_wgt + 3 * c, 24ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(P + c, d_P + c, 8ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(cell_id + 3 * c, d_cell + 3 * c, 24ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(pid + c, d_pid + c, 8ull * k, d2h, ctx->side);
      if (e == cudaSuccess) e = cudaMemcpyAsync(status + c, d_st + c, 8ull * k, d2h, ctx->side);
    }
    return e;
  };
  const bool pinned = ctx->xfer_route != FDF_TRANSFER_STAGED && host_views(arrays, views);
  int route = FDF_TRANSFER_STAGED;
  int64_t done = 0;
  cudaError_t e = cudaSuccess;
  if (pinned && ctx->xfer_route == FDF_TRANSFER_IN_PLACE) {
    route = FDF_TRANSFER_IN_PLACE;
  } else if (pinned && ctx->route_down >= 0) {
    route = ctx->route_down;
  } else if (pinned && xfer_slice(n) > 0) {
    route = calibrate_route(ctx, xfer_slice(n), run, done, e);
    if (e == cudaSuccess) ctx->route_down = route;
  }
  if (e == cudaSuccess) e = run(route == FDF_TRANSFER_IN_PLACE ? 1 : 0, done, n - done);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->side);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_GetSwarm: ") + cudaGetErrorString(e));
  return FDF_SUCCESS;
}

int fdf_GetScatteredFields(FdfContext *ctx, double *count, double *P_avg) {
  if (!ctx || !count || !P_avg) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetScatteredFields: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetScatteredFields: no grid");
  CU(cudaSetDevice(ctx->device));
  if (form_is32(ctx->out_form)) {
    launch_f32_to_f64(ctx->count32, ctx->count, ctx->g.Nn, ctx->stream);
    launch_f32_to_f64(ctx->avg32, ctx->avg, ctx->g.Nn, ctx->stream);
    CHECK_LAUNCH();
  }
  CU(cudaMemcpyAsync(count, ctx->count, 8ull * ctx->g.Nn, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaMemcpyAsync(P_avg, ctx->avg, 8ull * ctx->g.Nn, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

int fdf_GetCornerField(FdfContext *ctx, double *corner) {
  if (!ctx || !corner) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetCornerField: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetCornerField: no grid");
  if (!ctx->has_ucat) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetCornerField: no ucat");
  CU(cudaSetDevice(ctx->device));
  // the step computes only the nodes next to occupied cells; the full field is made here
  launch_center_to_corner(ctx->ucat, ctx->g, ctx->corner, nullptr, nullptr, ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  std::vector<double> soa(3 * (size_t)ctx->g.Nn);
  CU(cudaMemcpyAsync(soa.data(), ctx->corner, 24ull * ctx->g.Nn, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  const long long Nn = ctx->g.Nn;
  for (long long q = 0; q < Nn; ++q) {
    corner[3 * q] = soa[q]; corner[3 * q + 1] = soa[Nn + q]; corner[3 * q + 2] = soa[2 * Nn + q];
  }
  return FDF_SUCCESS;
}

int fdf_GetFaceDeposits(FdfContext *ctx, double *fi, double *fj, double *fk) {
  if (!ctx || !fi || !fj || !fk) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetFaceDeposits: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetFaceDeposits: no grid");
  const GridDims &g = ctx->g;
  long long nfi = (g.IM + 1LL) * g.JM * g.KM, nfj = g.IM * (g.JM + 1LL) * g.KM, nfk = (long long)g.IM * g.JM * (g.KM + 1LL);
  CU(cudaSetDevice(ctx->device));
  if (form_is32(ctx->out_form)) {
    launch_f32_to_f64(ctx->fi32, ctx->fi, nfi, ctx->stream);
    launch_f32_to_f64(ctx->fj32, ctx->fj, nfj, ctx->stream);
    launch_f32_to_f64(ctx->fk32, ctx->fk, nfk, ctx->stream);
    CHECK_LAUNCH();
  }
  CU(cudaMemcpyAsync(fi, ctx->fi, 8ull * nfi, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaMemcpyAsync(fj, ctx->fj, 8ull * nfj, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaMemcpyAsync(fk, ctx->fk, 8ull * nfk, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

}  // extern "C"

namespace {

// Kernels one pipeline run launches: locate, 3 scan kernels, corner, slots, order, gather,
// deposit; the learned form adds the flag scan (3), the compaction, the network and the walk
// from P1.
long long launches_per_step(const FdfContext *ctx) {
  return 10 + (ctx->swarm_form == FDF_FORM_LEARNED_FP32 ? 6 : 0);
}

// The shared pipeline of the initial setup (advect=0, drop=0) and a step (1, 1); locate_only:
// the walk and the re-sort alone (fdf_LocateAllParticlesInGrid), no interpolation or deposit.
int run_pipeline(FdfContext *ctx, int advect, int drop, FdfStepInfo *info, bool locate_only = false) {
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no grid: call fdf_SetGrid first");
  if (!ctx->has_ucat) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no ucat: call fdf_SetUcat first");
  if (!ctx->swarm_set) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no swarm: call fdf_SetSwarm first");
  CU(cudaSetDevice(ctx->device));
  if (ctx->swarm_form == FDF_FORM_LEARNED_FP32) {
    if (!ctx->loc.has_params)
      return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "learned form: no locator (fdf_LocatorTrain or fdf_LocatorSetParams)");
    int r = locator_reserve(ctx);
    if (r) return r;
  }
  cudaStream_t s = ctx->stream;
  const GridDims &g = ctx->g;
  int n_start = 0;
  if (info) {
    CU(cudaMemcpyAsync(&n_start, &ctx->cnt->n_sorted, sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  // zero the per-step counters; the error word stays set until the swarm is replaced
  CU(cudaMemsetAsync(ctx->cnt, 0, offsetof(DevCounters, err), s));
  CU(cudaMemsetAsync(ctx->cell_start, 0, 4ull * (g.Nc + 2), s));
  const bool prof = ctx->profiling;
  SwarmBuf &src = ctx->buf[ctx->cur];
  SwarmBuf &dst = ctx->buf[1 - ctx->cur];
  const bool f32 = form_is32(ctx->swarm_form);
  const bool learned = ctx->swarm_form == FDF_FORM_LEARNED_FP32;
  size_t e0 = prof ? record_event(ctx, s) : 0, eg0 = 0, eg1 = 0;
  if (learned) {
    // one evaluation in the previous cell; the particles that left it for a cell at least
    // far_cells away get a learned guess, and the reference walk from P1 (k_locate32_path)
    // fetches the rows of the path toward the guess ahead of its evaluations
    LocatorState &L = ctx->loc;
    launch_locate32(src, ctx->cap, g, ctx->table32, ctx->planes, ctx->dt, advect, ctx->bbox, ctx->fbox, drop,
                    ctx->cnt, ctx->keys, ctx->rank, ctx->cell_start, ctx->sentinel, L.pflag, L.far_cells, s);
    const long long nw = ((long long)ctx->cap + 31) / 32;   // the warps' pending counts, scanned in place
    exclusive_scan_u32(L.pflag + nw, nw + 1, L.scan_sums, s);
    launch_compact_pending(L.pflag, ctx->cap, L.pending, ctx->cnt, s);
    eg0 = prof ? record_event(ctx, s) : 0;
    mlp_guess_tc(L.tc_img, L.infer_bf16, L.bias, L.norm, src.x, src.y, src.z, 1, L.pending, &ctx->cnt->pending, 0,
                 ctx->cap, g, L.guess, ctx->num_sms, &ctx->cnt->err, s);
    eg1 = prof ? record_event(ctx, s) : 0;
    launch_locate32_path(src, ctx->cap, g, ctx->table32, ctx->planes, ctx->bbox, ctx->fbox, drop, ctx->cnt,
                         ctx->keys, ctx->rank, ctx->cell_start, ctx->sentinel, L.pending, L.guess, ctx->num_sms, s);
  } else if (f32) {
    launch_locate32(src, ctx->cap, g, ctx->table32, ctx->planes, ctx->dt, advect, ctx->bbox, ctx->fbox, drop,
                    ctx->cnt, ctx->keys, ctx->rank, ctx->cell_start, ctx->sentinel, nullptr, 0.f, s);
  } else {
    launch_locate(src, ctx->cap, g, ctx->table32, ctx->planes, ctx->dt, advect, ctx->bbox, drop, ctx->cnt,
                    ctx->keys, ctx->rank, ctx->cell_start, ctx->sentinel, s);
  }
  size_t e1 = prof ? record_event(ctx, s) : 0;
  exclusive_scan_u32(ctx->cell_start, g.Nc + 2, ctx->scan_sums, s);
  // the corner field needs only cell_start: compute it beside the slot assignment
  size_t c0 = 0, c1 = 0;
  if (!locate_only) {
    CU(cudaEventRecord(ctx->ev_scan, s));
    CU(cudaStreamWaitEvent(ctx->side, ctx->ev_scan, 0));
    c0 = prof ? record_event(ctx, ctx->side) : 0;
    if (f32)   // FP32 arithmetic is cheap: every node, no occupancy test
      launch_center_to_corner32(ctx->ucat32, g, ctx->corner32, nullptr, nullptr, ctx->side);
    else
      launch_center_to_corner(ctx->ucat, g, ctx->corner, ctx->cell_start, &ctx->cnt->nodes_total, ctx->side);
    c1 = prof ? record_event(ctx, ctx->side) : 0;
    CU(cudaEventRecord(ctx->ev_corner, ctx->side));
  }
  launch_scatter_slots(ctx->keys, ctx->rank, ctx->cap, ctx->cnt, ctx->sentinel, drop ? 0 : 1, ctx->cell_start,
                       ctx->perm, s);
  // the plain form orders each cell by PID (the oracle's summation order); the precision forms
  // keep each cell's particles in their previous order (no gather of the PIDs)
  launch_order_segments(ctx->cell_start, (int)(g.Nc + 1), f32 ? nullptr : src.pid, ctx->perm, s);
  size_t e2 = prof ? record_event(ctx, s) : 0;
  if (!locate_only) CU(cudaStreamWaitEvent(s, ctx->ev_corner, 0));
  size_t e3 = prof ? record_event(ctx, s) : 0;
  const int gmode = locate_only ? GATHER_COPY : GATHER_INTERP;
  if (f32)
    launch_gather_interp32(src, dst, ctx->cap, g, ctx->corner32, ctx->perm, ctx->cell_start, ctx->cnt, s, gmode);
  else
    launch_gather_interp(src, dst, ctx->cap, g, ctx->corner, ctx->perm, ctx->cell_start, ctx->cnt, s, gmode);
  size_t e4 = prof ? record_event(ctx, s) : 0;
  const long long nfi = (g.IM + 1LL) * g.JM * g.KM, nfj = g.IM * (g.JM + 1LL) * g.KM;
  if (locate_only) {
    // no deposit
  } else if (f32) {
    float *m = ctx->momentum ? ctx->mom32 : nullptr;
    launch_deposit32(dst, g, ctx->cell_start, ctx->volume, ctx->count32, ctx->avg32, ctx->fi32, ctx->fj32, ctx->fk32,
                     m, m ? m + 3 * nfi : nullptr, m ? m + 3 * (nfi + nfj) : nullptr, s);
  } else {
    double *m = ctx->momentum ? ctx->mom : nullptr;
    launch_deposit(dst, g, ctx->cell_start, ctx->volume, ctx->count, ctx->avg, ctx->fi, ctx->fj, ctx->fk, m,
                   m ? m + 3 * nfi : nullptr, m ? m + 3 * (nfi + nfj) : nullptr, s);
  }
  launch_fold_counts(ctx->cnt, s);
  ctx->out_momentum = ctx->momentum;
  ctx->out_form = ctx->swarm_form;
  size_t e5 = prof ? record_event(ctx, s) : 0;
  if (prof && learned) {
    ctx->ev_spans.push_back({FDF_STAGE_LOCATE, {e0, eg0}});
    ctx->ev_spans.push_back({FDF_STAGE_GUESS, {eg0, eg1}});
    ctx->ev_spans.push_back({FDF_STAGE_GUESS_WALK, {eg1, e1}});
  } else if (prof) {
    ctx->ev_spans.push_back({FDF_STAGE_LOCATE, {e0, e1}});
  }
  if (prof) {
    ctx->ev_spans.push_back({FDF_STAGE_SORT, {e1, e2}});
    if (!locate_only) {
      ctx->ev_spans.push_back({FDF_STAGE_CORNER, {c0, c1}});
      ctx->ev_spans.push_back({FDF_STAGE_WAIT, {e2, e3}});
    }
    ctx->ev_spans.push_back({FDF_STAGE_GATHER_INTERP, {e3, e4}});
    if (!locate_only) ctx->ev_spans.push_back({FDF_STAGE_DEPOSIT, {e4, e5}});
  }
  CHECK_LAUNCH();
  ctx->cur = 1 - ctx->cur;
  ctx->layout_ok = true;
  ctx->launches += launches_per_step(ctx) - (locate_only ? 2 : 0);
  if (info) {
    DevCounters c{};
    CU(cudaMemcpyAsync(&c, ctx->cnt, DEVCOUNTERS_HEAD, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    info->n_start = n_start;
    info->n_end = c.n_sorted;
    info->removed_lost = (int64_t)c.removed_lost;
    info->removed_oob = (int64_t)c.removed_oob;
    info->walk_evals = (int64_t)c.evals;
    info->fp64_fallbacks = (int64_t)c.fallbacks;
    if (c.err & ERRBIT_DEGENERATE)
      return fail(ctx, FDF_ERR_USER, "Degenerate plane detected (normal vector is near zero).");
    if (c.err & ERRBIT_TC_TIMEOUT) return fail(ctx, FDF_ERR_GPU, "learned locator: tensor-core wait timed out");
  }
  return FDF_SUCCESS;
}

// Re-sorts the held particles by cell -- within a cell by PID in the plain form, in their
// previous order in the precision forms -- into the other buffer, dropping the LOST and/or the
// out-of-bounds ones; cell_start then matches the held particles.
int resort(FdfContext *ctx, int remove_lost, int remove_oob, int64_t *removed_lost, int64_t *removed_oob) {
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no grid: call fdf_SetGrid first");
  if (!ctx->swarm_set) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no swarm: call fdf_SetSwarm first");
  CU(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const GridDims &g = ctx->g;
  const bool f32 = form_is32(ctx->swarm_form);
  SwarmBuf &src = ctx->buf[ctx->cur];
  SwarmBuf &dst = ctx->buf[1 - ctx->cur];
  CU(cudaMemsetAsync(ctx->cnt, 0, offsetof(DevCounters, err), s));
  CU(cudaMemsetAsync(ctx->cell_start, 0, 4ull * (g.Nc + 2), s));
  launch_resort_keys(src, ctx->cap, g, f32 ? 1 : 0, remove_lost, remove_oob, ctx->bbox, ctx->fbox, ctx->cnt,
                     ctx->keys, ctx->rank, ctx->cell_start, ctx->sentinel, s);
  exclusive_scan_u32(ctx->cell_start, g.Nc + 2, ctx->scan_sums, s);
  launch_scatter_slots(ctx->keys, ctx->rank, ctx->cap, ctx->cnt, ctx->sentinel, 1, ctx->cell_start, ctx->perm, s);
  launch_order_segments(ctx->cell_start, (int)(g.Nc + 1), f32 ? nullptr : src.pid, ctx->perm, s);
  if (f32)
    launch_gather_interp32(src, dst, ctx->cap, g, ctx->corner32, ctx->perm, ctx->cell_start, ctx->cnt, s, GATHER_COPY);
  else
    launch_gather_interp(src, dst, ctx->cap, g, ctx->corner, ctx->perm, ctx->cell_start, ctx->cnt, s, GATHER_COPY);
  launch_fold_counts(ctx->cnt, s);
  CHECK_LAUNCH();
  ctx->launches += 8;
  ctx->cur = 1 - ctx->cur;
  ctx->layout_ok = true;
  DevCounters c{};
  CU(cudaMemcpyAsync(&c, ctx->cnt, DEVCOUNTERS_HEAD, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if (removed_lost) *removed_lost = (int64_t)c.removed_lost;
  if (removed_oob) *removed_oob = (int64_t)c.removed_oob;
  return FDF_SUCCESS;
}

int ensure_layout(FdfContext *ctx) { return ctx->layout_ok ? FDF_SUCCESS : resort(ctx, 0, 0, nullptr, nullptr); }

}  // namespace

extern "C" {

int fdf_ResetAllParticleStatuses(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->swarm_set) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no swarm: call fdf_SetSwarm first");
  CU(cudaSetDevice(ctx->device));
  launch_reset_status(ctx->buf[ctx->cur], ctx->cap, ctx->cnt, ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  return FDF_SUCCESS;
}

int fdf_UpdateAllParticlePositions(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->swarm_set) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no swarm: call fdf_SetSwarm first");
  CU(cudaSetDevice(ctx->device));
  if (form_is32(ctx->swarm_form))
    launch_advect32(ctx->buf[ctx->cur], ctx->cap, ctx->dt, ctx->cnt, ctx->stream);
  else
    launch_advect(ctx->buf[ctx->cur], ctx->cap, ctx->dt, ctx->cnt, ctx->stream);
  CHECK_LAUNCH();
  ctx->launches += 1;
  return FDF_SUCCESS;
}

int fdf_LocateAllParticlesInGrid(FdfContext *ctx, FdfStepInfo *info) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  FdfStepInfo local{};
  return run_pipeline(ctx, 0, 0, info ? info : &local, true);
}

int fdf_CheckAndRemoveLostParticles(FdfContext *ctx, int64_t *removed) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  return resort(ctx, 1, 0, removed, nullptr);
}

int fdf_CheckAndRemoveOutOfBoundsParticles(FdfContext *ctx, int64_t *removed) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  return resort(ctx, 0, 1, nullptr, removed);
}

int fdf_InterpolateAllFieldsToSwarm(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_ucat) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "no ucat: call fdf_SetUcat first");
  int r = ensure_layout(ctx);
  if (r) return r;
  const GridDims &g = ctx->g;
  SwarmBuf &b = ctx->buf[ctx->cur];
  if (form_is32(ctx->swarm_form)) {
    launch_center_to_corner32(ctx->ucat32, g, ctx->corner32, nullptr, nullptr, ctx->stream);
    launch_gather_interp32(b, b, ctx->cap, g, ctx->corner32, nullptr, ctx->cell_start, ctx->cnt, ctx->stream,
                           INTERP_KEEP);
  } else {
    launch_center_to_corner(ctx->ucat, g, ctx->corner, ctx->cell_start, &ctx->cnt->nodes_total, ctx->stream);
    launch_gather_interp(b, b, ctx->cap, g, ctx->corner, nullptr, ctx->cell_start, ctx->cnt, ctx->stream,
                         INTERP_KEEP);
  }
  CHECK_LAUNCH();
  ctx->launches += 2;
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

int fdf_ScatterAllParticleFieldsToEulerFields(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  int r = ensure_layout(ctx);
  if (r) return r;
  const GridDims &g = ctx->g;
  SwarmBuf &b = ctx->buf[ctx->cur];
  const long long nfi = (g.IM + 1LL) * g.JM * g.KM, nfj = g.IM * (g.JM + 1LL) * g.KM;
  if (form_is32(ctx->swarm_form)) {
    float *m = ctx->momentum ? ctx->mom32 : nullptr;
    launch_deposit32(b, g, ctx->cell_start, ctx->volume, ctx->count32, ctx->avg32, ctx->fi32, ctx->fj32, ctx->fk32,
                     m, m ? m + 3 * nfi : nullptr, m ? m + 3 * (nfi + nfj) : nullptr, ctx->stream);
  } else {
    double *m = ctx->momentum ? ctx->mom : nullptr;
    launch_deposit(b, g, ctx->cell_start, ctx->volume, ctx->count, ctx->avg, ctx->fi, ctx->fj, ctx->fk, m,
                   m ? m + 3 * nfi : nullptr, m ? m + 3 * (nfi + nfj) : nullptr, ctx->stream);
  }
  CHECK_LAUNCH();
  ctx->launches += 1;
  ctx->out_momentum = ctx->momentum;
  ctx->out_form = ctx->swarm_form;
  CU(cudaStreamSynchronize(ctx->stream));
  return FDF_SUCCESS;
}

int fdf_LocatePoints(FdfContext *ctx, int64_t n, const double *position, const int64_t *cell_in, int64_t *cell_out,
                     double *weight, int64_t *status) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (n > 0 && (!position || !cell_out || !weight || !status))
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_LocatePoints: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_LocatePoints: call fdf_SetGrid first");
  if (n < 0 || n > FDF_MAX_PARTICLES) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_LocatePoints: n out of range");
  if (n == 0) return FDF_SUCCESS;
  CU(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const GridDims &g = ctx->g;
  const int m = (int)n;
  // the points as a temporary plain-form swarm: NEEDS_LOCATION, walk start = the given cell
  void *mem = nullptr;
  const size_t sw = swarm_bytes_per_buf(m), aos = 24ull * m, one = 8ull * m;
  const size_t bytes = sw + 4 * aos + 3 * one + 4ull * m + 4ull * (g.Nc + 2) + sizeof(DevCounters) + 256 * 12;
  CU(cudaMalloc(&mem, bytes));
  char *p = (char *)mem;
  SwarmBuf tb;
  carve_swarm(p, m, tb);
  auto take = [&](size_t nb) { char *q = p; p += (nb + 255) / 256 * 256; return q; };
  take(sw);
  double *d_pos = (double *)take(aos);
  long long *d_cell = (long long *)take(aos);
  double *d_zero = (double *)take(aos);   // velocity, weight, P, pid, status (0 = NEEDS_LOCATION)
  double *d_w = (double *)take(aos);
  double *d_P = (double *)take(one);
  long long *d_pid = (long long *)take(one);
  long long *d_st = (long long *)take(one);
  unsigned int *keys = (unsigned int *)take(4ull * m);
  unsigned int *hist = (unsigned int *)take(4ull * (g.Nc + 2));
  DevCounters *tc = (DevCounters *)take(sizeof(DevCounters));
  DevCounters c0{};
  c0.n = m;
  c0.n_sorted = m;
  cudaError_t e = cudaMemcpyAsync(d_pos, position, aos, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cell_in ? cudaMemcpyAsync(d_cell, cell_in, aos, cudaMemcpyHostToDevice, s) : cudaMemsetAsync(d_cell, 0xff, aos, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_zero, 0, aos, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, 4ull * (g.Nc + 2), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tc, &c0, sizeof(c0), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    launch_swarm_from_aos(d_pos, d_zero, d_zero, d_zero, d_cell, (const long long *)d_zero, (const long long *)d_zero,
                          m, g, tb, s);
    launch_locate(tb, m, g, ctx->table32, ctx->planes, 0.0, 0, ctx->bbox, 0, tc, keys, nullptr, hist, ctx->sentinel,
                    s);
    launch_swarm_to_aos(tb, m, g, d_pos, d_zero, d_w, d_P, d_cell, d_pid, d_st, s);
    ctx->launches += 3;
    e = cudaGetLastError();
  }
  unsigned int err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(cell_out, d_cell, aos, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(weight, d_w, aos, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(status, d_st, one, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &tc->err, sizeof(err), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(mem);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_LocatePoints: ") + cudaGetErrorString(e));
  if (err & ERRBIT_DEGENERATE) return fail(ctx, FDF_ERR_USER, "Degenerate plane detected (normal vector is near zero).");
  return FDF_SUCCESS;
}

int fdf_InterpolatePoints(FdfContext *ctx, int64_t n, const int64_t *cell, const double *weight, double *velocity) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (n > 0 && (!cell || !weight || !velocity)) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_InterpolatePoints: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_InterpolatePoints: call fdf_SetGrid first");
  if (!ctx->has_ucat) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_InterpolatePoints: call fdf_SetUcat first");
  if (n < 0 || n > FDF_MAX_PARTICLES) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_InterpolatePoints: n out of range");
  if (n == 0) return FDF_SUCCESS;
  CU(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const GridDims &g = ctx->g;
  const int m = (int)n;
  // the points as a temporary plain-form swarm in their own order (no sort): cells and weights
  // in, velocities out; cell_start only carries the count the gather reads at [Nc], [Nc + 1]
  void *mem = nullptr;
  const size_t sw = swarm_bytes_per_buf(m), aos = 24ull * m, one = 8ull * m;
  const size_t bytes = sw + 4 * aos + 3 * one + 4ull * (g.Nc + 2) + sizeof(DevCounters) + 256 * 10;
  CU(cudaMalloc(&mem, bytes));
  char *p = (char *)mem;
  SwarmBuf tb;
  carve_swarm(p, m, tb);
  auto take = [&](size_t nb) { char *q = p; p += (nb + 255) / 256 * 256; return q; };
  take(sw);
  double *d_w = (double *)take(aos);
  long long *d_cell = (long long *)take(aos);
  double *d_zero = (double *)take(aos);     // position, velocity, P, pid, status (0 = NEEDS_LOCATION)
  double *d_vel = (double *)take(aos);
  double *d_P = (double *)take(one);
  long long *d_pid = (long long *)take(one);
  long long *d_st = (long long *)take(one);
  unsigned int *cs = (unsigned int *)take(4ull * (g.Nc + 2));
  DevCounters *tc = (DevCounters *)take(sizeof(DevCounters));
  const unsigned int counts[2] = {(unsigned int)m, (unsigned int)m};
  cudaError_t e = cudaMemcpyAsync(d_w, weight, aos, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_cell, cell, aos, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_zero, 0, aos, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cs + g.Nc, counts, sizeof(counts), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(tc, 0, sizeof(DevCounters), s);
  if (e == cudaSuccess) {
    // every node of the corner field (the swarm steps compute only the nodes they need)
    launch_center_to_corner(ctx->ucat, g, ctx->corner, nullptr, nullptr, s);
    launch_swarm_from_aos(d_zero, d_zero, d_w, d_zero, d_cell, (const long long *)d_zero, (const long long *)d_zero,
                          m, g, tb, s);
    launch_gather_interp(tb, tb, m, g, ctx->corner, nullptr, cs, tc, s, INTERP_KEEP);
    launch_swarm_to_aos(tb, m, g, d_zero, d_vel, d_w, d_P, d_cell, d_pid, d_st, s);
    ctx->launches += 4;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(velocity, d_vel, aos, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(mem);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_InterpolatePoints: ") + cudaGetErrorString(e));
  return FDF_SUCCESS;
}

// ---- k-slab decomposition over several ranks (a driver that splits the swarm over GPUs) ----

int fdf_ExtractParticles(FdfContext *ctx, int64_t k_lo, int64_t k_hi, int64_t n_max, int64_t *n_out,
                         double *position, double *velocity, double *weight, double *P, int64_t *cell_id,
                         int64_t *pid, int64_t *status) {
  if (!ctx || !n_out) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_ExtractParticles: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_ExtractParticles: call fdf_SetGrid first");
  if (k_lo < 0 || k_hi < k_lo || k_hi > ctx->g.KM)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_ExtractParticles: need 0 <= k_lo <= k_hi <= KM");
  int r = ensure_layout(ctx);   // sorted by (cell, PID): the slab is one contiguous range
  if (r) return r;
  const GridDims &g = ctx->g;
  const long long L = (long long)g.IM * g.JM;
  unsigned int bound[3] = {0, 0, 0};
  int n_held = 0;
  cudaStream_t s = ctx->stream;
  CU(cudaMemcpyAsync(&bound[0], ctx->cell_start + k_lo * L, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&bound[1], ctx->cell_start + k_hi * L, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&bound[2], ctx->cell_start + g.Nc, 4, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(&n_held, &ctx->cnt->n_sorted, sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const int a = (int)bound[0], b = (int)bound[1], c = (int)bound[2], n = n_held;
  const int64_t m = (int64_t)a + (c - b);   // cells below the slab, then above it
  *n_out = m;
  if (m > n_max) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_ExtractParticles: output arrays too small");
  if (m == 0) return FDF_SUCCESS;
  if (!position || !velocity || !weight || !P || !cell_id || !pid || !status)
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_ExtractParticles: null field pointer");
  const bool f32 = form_is32(ctx->swarm_form);
  double *d_pos = (double *)ctx->staging, *d_vel = d_pos + 3 * m, *d_wgt = d_vel + 3 * m, *d_P = d_wgt + 3 * m;
  long long *d_cell = (long long *)(d_P + m), *d_pid = d_cell + 3 * m, *d_st = d_pid + m;
  const int ranges[2][2] = {{0, a}, {b, c}};
  long long o = 0;
  for (int q = 0; q < 2; ++q) {
    const int r0 = ranges[q][0], cnt = ranges[q][1] - ranges[q][0];
    if (cnt <= 0) continue;
    const SwarmBuf src = shifted(ctx->buf[ctx->cur], r0);
    if (f32)
      launch_swarm_to_aos32(src, cnt, g, d_pos + 3 * o, d_vel + 3 * o, d_wgt + 3 * o, d_P + o, d_cell + 3 * o,
                            d_pid + o, d_st + o, s);
    else
      launch_swarm_to_aos(src, cnt, g, d_pos + 3 * o, d_vel + 3 * o, d_wgt + 3 * o, d_P + o, d_cell + 3 * o,
                          d_pid + o, d_st + o, s);
    ctx->launches += 1;
    o += cnt;
  }
  CHECK_LAUNCH();
  CU(cudaMemcpyAsync(position, d_pos, 24ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(velocity, d_vel, 24ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(weight, d_wgt, 24ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(P, d_P, 8ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(cell_id, d_cell, 24ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(pid, d_pid, 8ull * m, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(status, d_st, 8ull * m, cudaMemcpyDeviceToHost, s));
  // the rest stays, in its sorted order: the slab's cells, then the particles without a cell
  launch_move_kept(ctx->buf[ctx->cur], ctx->buf[1 - ctx->cur], a, b, c, n, s);
  CHECK_LAUNCH();
  ctx->launches += 1;
  const int kept = n - (int)m;
  CU(cudaMemcpyAsync(&ctx->cnt->n, &kept, sizeof(int), cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(&ctx->cnt->n_sorted, &kept, sizeof(int), cudaMemcpyHostToDevice, s));
  CU(cudaStreamSynchronize(s));
  ctx->cur = 1 - ctx->cur;
  ctx->layout_ok = false;   // cell_start no longer matches the held slots
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_AddParticles(FdfContext *ctx, int64_t n, const double *position, const double *velocity,
                     const double *weight, const double *P, const int64_t *cell_id, const int64_t *pid,
                     const int64_t *status) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (n < 0) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_AddParticles: negative count");
  if (n == 0) return FDF_SUCCESS;
  if (!position || !velocity || !weight || !P || !cell_id || !pid || !status)
    return fail(ctx, FDF_ERR_ARG_NULL, "fdf_AddParticles: null field pointer");
  if (!ctx->swarm_set) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_AddParticles: no swarm (fdf_SetSwarm first)");
  CU(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  int n_held = 0;
  CU(cudaMemcpyAsync(&n_held, &ctx->cnt->n_sorted, sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if ((long long)n_held + n > ctx->cap)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE,
                "fdf_AddParticles: the swarm would exceed its capacity (fdf_ReserveParticles before fdf_SetSwarm)");
  double *d_pos = (double *)ctx->staging, *d_vel = d_pos + 3 * n, *d_wgt = d_vel + 3 * n, *d_P = d_wgt + 3 * n;
  long long *d_cell = (long long *)(d_P + n), *d_pid = d_cell + 3 * n, *d_st = d_pid + n;
  CU(cudaMemcpyAsync(d_pos, position, 24ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_vel, velocity, 24ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_wgt, weight, 24ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_P, P, 8ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_cell, cell_id, 24ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_pid, pid, 8ull * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(d_st, status, 8ull * n, cudaMemcpyHostToDevice, s));
  const SwarmBuf dst = shifted(ctx->buf[ctx->cur], n_held);
  if (form_is32(ctx->swarm_form))
    launch_swarm_from_aos32(d_pos, d_vel, d_wgt, d_P, d_cell, d_pid, d_st, (int)n, ctx->g, dst, s);
  else
    launch_swarm_from_aos(d_pos, d_vel, d_wgt, d_P, d_cell, d_pid, d_st, (int)n, ctx->g, dst, s);
  CHECK_LAUNCH();
  ctx->launches += 1;
  const int total = n_held + (int)n;
  CU(cudaMemcpyAsync(&ctx->cnt->n, &total, sizeof(int), cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(&ctx->cnt->n_sorted, &total, sizeof(int), cudaMemcpyHostToDevice, s));
  CU(cudaStreamSynchronize(s));
  ctx->layout_ok = false;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_DepositKFaceLayer(FdfContext *ctx, int64_t k, const double *seed, const double *seed_momentum) {
  if (!ctx || !seed) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_DepositKFaceLayer: null argument");
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_DepositKFaceLayer: call fdf_SetGrid first");
  if (k < 0 || k > ctx->g.KM) return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_DepositKFaceLayer: need 0 <= k <= KM");
  if (ctx->out_form != FDF_FORM_PLAIN_FP64 || ctx->swarm_form != FDF_FORM_PLAIN_FP64)
    return fail(ctx, FDF_ERR_SUP, "fdf_DepositKFaceLayer: the plain FP64 form's deposits only");
  if (!ctx->layout_ok)
    return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_DepositKFaceLayer: deposit the held particles first");
  CU(cudaSetDevice(ctx->device));
  const GridDims &g = ctx->g;
  const long long L = (long long)g.IM * g.JM;
  const bool mom = ctx->out_momentum && ctx->mom;
  double *d = nullptr;
  CU(cudaMalloc((void **)&d, 8ull * L * 4));
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(d, seed, 8ull * L, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = seed_momentum ? cudaMemcpyAsync(d + L, seed_momentum, 24ull * L, cudaMemcpyHostToDevice, s)
                      : cudaMemsetAsync(d + L, 0, 24ull * L, s);
  const long long nfi = (g.IM + 1LL) * g.JM * g.KM, nfj = g.IM * (g.JM + 1LL) * g.KM;
  if (e == cudaSuccess) {
    launch_deposit_k_layer(ctx->buf[ctx->cur], g, ctx->cell_start, (int)k, ctx->volume, d, d + L, ctx->fk,
                           mom ? ctx->mom + 3 * (nfi + nfj) : nullptr, s);
    ctx->launches += 1;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("fdf_DepositKFaceLayer: ") + cudaGetErrorString(e));
  return FDF_SUCCESS;
}

int fdf_PerformInitialSetup(FdfContext *ctx, FdfStepInfo *info) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  FdfStepInfo local{};
  return run_pipeline(ctx, 0, 0, info ? info : &local);
}

int fdf_AdvanceStep(FdfContext *ctx, FdfStepInfo *info) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  return run_pipeline(ctx, 1, 1, info);
}

// nsteps steps without host round trips.  Unless stage timing is on, each step replays a
// CUDA graph of the step captured for the current swarm buffer parity (the first step after
// any change runs eagerly, then the graph is captured from the next one); a launch-bound
// small swarm then pays one graph launch per step instead of a dozen kernel launches.
int fdf_AdvanceSteps(FdfContext *ctx, int nsteps) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  for (int q = 0; q < nsteps; ++q) {
    const int parity = ctx->cur;
    if (ctx->profiling || ctx->eager_gen != ctx->gen) {
      // eager: stage timing, or the first step after a change (one-time set-up stays out of capture)
      int r = run_pipeline(ctx, 1, 1, nullptr);
      if (r) return r;
      ctx->eager_gen = ctx->gen;
      continue;
    }
    if (ctx->graph_gen[parity] != ctx->gen || !ctx->step_graph[parity]) {
      CU(cudaSetDevice(ctx->device));
      if (ctx->step_graph[parity]) { cudaGraphExecDestroy(ctx->step_graph[parity]); ctx->step_graph[parity] = nullptr; }
      const long long launches0 = ctx->launches;
      CU(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
      const int r = run_pipeline(ctx, 1, 1, nullptr);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
      ctx->cur = parity;                 // the capture ran nothing: restore the host state
      ctx->launches = launches0;
      if (r) { if (graph) cudaGraphDestroy(graph); return r; }
      if (e != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("step capture: ") + cudaGetErrorString(e));
      const cudaError_t ei = cudaGraphInstantiate(&ctx->step_graph[parity], graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) return fail(ctx, FDF_ERR_GPU, std::string("step graph: ") + cudaGetErrorString(ei));
      ctx->graph_gen[parity] = ctx->gen;
    }
    CU(cudaGraphLaunch(ctx->step_graph[parity], ctx->stream));
    ctx->cur = 1 - parity;
    ctx->out_form = ctx->swarm_form;
    ctx->out_momentum = ctx->momentum;
    ctx->launches += launches_per_step(ctx);
  }
  return FDF_SUCCESS;
}

int fdf_Synchronize(FdfContext *ctx) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  CU(cudaSetDevice(ctx->device));
  CU(cudaStreamSynchronize(ctx->stream));
  unsigned int err = 0;
  CU(cudaMemcpy(&err, &ctx->cnt->err, sizeof(err), cudaMemcpyDeviceToHost));
  if (err & ERRBIT_DEGENERATE) return fail(ctx, FDF_ERR_USER, "Degenerate plane detected (normal vector is near zero).");
  if (err & ERRBIT_TC_TIMEOUT) return fail(ctx, FDF_ERR_GPU, "learned locator: tensor-core wait timed out");
  return FDF_SUCCESS;
}

void *fdf_GetStream(FdfContext *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

const char *fdf_GetLastError(FdfContext *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int64_t fdf_GetLaunchCount(FdfContext *ctx) { return ctx ? ctx->launches : 0; }

int fdf_GetCounters(FdfContext *ctx, int64_t *particle_steps, int64_t *walk_evals, int64_t *corner_nodes) {
  if (!ctx || !particle_steps || !walk_evals || !corner_nodes) return FDF_ERR_ARG_NULL;
  CU(cudaSetDevice(ctx->device));
  DevCounters c{};
  CU(cudaMemcpyAsync(&c, ctx->cnt, DEVCOUNTERS_HEAD, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  *particle_steps = (int64_t)c.psteps_total;
  *walk_evals = (int64_t)c.evals_total;
  *corner_nodes = (int64_t)c.nodes_total;
  return FDF_SUCCESS;
}

int fdf_SortByCell(const int32_t *cell_ids, int64_t n, int64_t ncells, uint32_t *perm, uint32_t *cell_start,
                   void *stream) {
  if (n > 0 && (!cell_ids || !perm)) return FDF_ERR_ARG_NULL;
  if (!cell_start) return FDF_ERR_ARG_NULL;
  if (n < 0 || n > FDF_MAX_PARTICLES || ncells < 1 || ncells + 1 > scan_max_count()) return FDF_ERR_ARG_OUTOFRANGE;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *cursor = nullptr, *sums = nullptr;
  const size_t nsums = scan_scratch_words(ncells + 1);
  if (cudaMallocAsync((void **)&cursor, 4ull * ncells, s) != cudaSuccess) return FDF_ERR_MEM;
  if (cudaMallocAsync((void **)&sums, 4ull * nsums, s) != cudaSuccess) {
    cudaFreeAsync(cursor, s);
    return FDF_ERR_MEM;
  }
  cell_sort_on_scratch(cell_ids, n, ncells, perm, cell_start, cursor, sums, s);
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(sums, s);
  cudaFreeAsync(cursor, s);
  return e == cudaSuccess ? FDF_SUCCESS : FDF_ERR_GPU;
}

int fdf_SetProfiling(FdfContext *ctx, int enable) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  CU(cudaSetDevice(ctx->device));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->profiling = enable != 0;
  ctx->gen++;
  ctx->ev_used = 0;
  ctx->ev_spans.clear();
  return FDF_SUCCESS;
}

int fdf_SetMomentumDeposit(FdfContext *ctx, int enable) {
  if (!ctx) return FDF_ERR_ARG_NULL;
  if (!ctx->has_grid) return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_SetMomentumDeposit: call fdf_SetGrid first");
  CU(cudaSetDevice(ctx->device));
  if (enable && (!ctx->mom || !ctx->mom32)) {
    const GridDims &g = ctx->g;
    const long long nf = (g.IM + 1LL) * g.JM * g.KM + g.IM * (g.JM + 1LL) * g.KM + (long long)g.IM * g.JM * (g.KM + 1LL);
    CU(cudaStreamSynchronize(ctx->stream));
    ctx->momentum = false;
    ctx->gen++;
    cfree(ctx->mom); cfree(ctx->mom32);
    CU(dev_alloc(&ctx->mom, 24ull * nf));
    CU(dev_alloc(&ctx->mom32, 12ull * nf));
    CU(cudaMemset(ctx->mom, 0, 24ull * nf));
    CU(cudaMemset(ctx->mom32, 0, 12ull * nf));
  }
  ctx->momentum = enable != 0;
  ctx->gen++;
  return FDF_SUCCESS;
}

int fdf_GetFaceMomentum(FdfContext *ctx, double *mi, double *mj, double *mk) {
  if (!ctx || !mi || !mj || !mk) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_GetFaceMomentum: null argument");
  if (!ctx->mom || !ctx->out_momentum)
    return fail(ctx, FDF_ERR_ARG_WRONGSTATE, "fdf_GetFaceMomentum: no momentum deposit (fdf_SetMomentumDeposit)");
  const GridDims &g = ctx->g;
  const long long nfs[3] = {(g.IM + 1LL) * g.JM * g.KM, g.IM * (g.JM + 1LL) * g.KM, (long long)g.IM * g.JM * (g.KM + 1LL)};
  const long long nf = nfs[0] + nfs[1] + nfs[2];
  CU(cudaSetDevice(ctx->device));
  if (form_is32(ctx->out_form)) {
    launch_f32_to_f64(ctx->mom32, ctx->mom, 3 * nf, ctx->stream);
    CHECK_LAUNCH();
    ctx->launches += 1;
  }
  std::vector<double> soa(3 * (size_t)nf);
  CU(cudaMemcpyAsync(soa.data(), ctx->mom, 24ull * nf, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  double *out[3] = {mi, mj, mk};
  size_t off = 0;
  for (int fam = 0; fam < 3; ++fam) {
    const long long n = nfs[fam];
    for (long long q = 0; q < n; ++q)
      for (int c = 0; c < 3; ++c) out[fam][3 * q + c] = soa[off + (size_t)c * n + q];
    off += 3 * (size_t)n;
  }
  return FDF_SUCCESS;
}

int fdf_GetStageTimes(FdfContext *ctx, double *ms_total, int64_t *launches, int nstages) {
  if (!ctx || !ms_total || !launches) return FDF_ERR_ARG_NULL;
  CU(cudaSetDevice(ctx->device));
  CU(cudaStreamSynchronize(ctx->stream));
  CU(cudaStreamSynchronize(ctx->side));
  for (int q = 0; q < nstages; ++q) { ms_total[q] = 0.0; launches[q] = 0; }
  for (auto &sp : ctx->ev_spans) {
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, ctx->ev_pool[sp.second.first], ctx->ev_pool[sp.second.second]));
    if (sp.first < nstages) { ms_total[sp.first] += ms; launches[sp.first] += 1; }
  }
  return FDF_SUCCESS;
}

}  // extern "C"
