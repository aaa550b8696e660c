// fdf_sort.cu -- per-step re-sort of the particles by cell.
//
// A stable LSD radix sort of (cell key, particle slot) pairs, 8 bits per pass,
// followed by a boundary fill that turns the sorted keys into cell_start[Nc+1]
// (the first sorted slot of every cell).  Removed particles carry the key Nc, so
// they sort to the end and cell_start[Nc] is the number of survivors: the sort
// is also the removal.  Stability makes the order -- and so every later sum --
// a deterministic function of the previous order.
//
// Per pass: (1) per-tile digit histogram, (2) exclusive scan of the digit-major
// histogram, (3) per-tile stable scatter.  In (3) each warp ranks its items in
// order with __match_any_sync and a per-warp digit counter in shared memory;
// the eight warps' counts are then scanned per digit.
#include "fdf_internal.cuh"

namespace {

constexpr int RADIX = 256;
constexpr int SORT_THREADS = 256;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int ITEMS = 16;
constexpr int TILE = SORT_THREADS * ITEMS;   // 4096
constexpr int WARP_CHUNK = TILE / SORT_WARPS;  // 512

__global__ void __launch_bounds__(SORT_THREADS) k_hist(const unsigned int *__restrict__ keys, const int *n_dev,
                                                      int shift, unsigned int *__restrict__ hist, int num_tiles) {
  __shared__ unsigned int cnt[RADIX];
  const int n = *n_dev;
  const int tile = blockIdx.x;
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) cnt[d] = 0;
  __syncthreads();
  const long long base = (long long)tile * TILE;
#pragma unroll 4
  for (int it = 0; it < ITEMS; ++it) {
    long long idx = base + it * SORT_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(__ldg(keys + idx) >> shift) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) hist[(long long)d * num_tiles + tile] = cnt[d];
}

// ---- exclusive scan of a u32 array (reduce -> scan sums -> scan with offsets) ----
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_BLOCK = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ unsigned int block_exclusive_scan(unsigned int v, unsigned int *total) {
  __shared__ unsigned int warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned int t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  unsigned int warp_prefix = wid ? warp_tot[wid - 1] : 0u;
  if (total) *total = warp_tot[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const unsigned int *__restrict__ in, long long count,
                                                             unsigned int *__restrict__ sums) {
  long long base = (long long)blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_ITEMS;
  unsigned int v = 0;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q)
    if (base + q < count) v += in[base + q];
  unsigned int tot;
  block_exclusive_scan(v, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Single block: exclusive scan of up to SCAN_THREADS*8 block sums in place.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(unsigned int *sums, int nsums) {
  constexpr int PER = 8;
  int base = threadIdx.x * PER;
  unsigned int v[PER], t = 0;
#pragma unroll
  for (int q = 0; q < PER; ++q) { v[q] = (base + q < nsums) ? sums[base + q] : 0u; t += v[q]; }
  unsigned int ex = block_exclusive_scan(t, nullptr);
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    if (base + q < nsums) sums[base + q] = ex;
    ex += v[q];
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(unsigned int *__restrict__ data, long long count,
                                                            const unsigned int *__restrict__ sums) {
  long long base = (long long)blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_ITEMS;
  unsigned int v[SCAN_ITEMS], t = 0;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q) { v[q] = (base + q < count) ? data[base + q] : 0u; t += v[q]; }
  unsigned int ex = block_exclusive_scan(t, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q) {
    if (base + q < count) data[base + q] = ex;
    ex += v[q];
  }
}

__global__ void __launch_bounds__(SORT_THREADS) k_scatter(const unsigned int *__restrict__ keys_in,
                                                         const unsigned int *__restrict__ vals_in,
                                                         unsigned int *__restrict__ keys_out,
                                                         unsigned int *__restrict__ vals_out, const int *n_dev,
                                                         int shift, const unsigned int *__restrict__ hist_scan,
                                                         int num_tiles) {
  __shared__ unsigned int wcnt[SORT_WARPS][RADIX];
  const int n = *n_dev;
  const int tile = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = threadIdx.x; q < SORT_WARPS * RADIX; q += SORT_THREADS) (&wcnt[0][0])[q] = 0;
  __syncthreads();
  const long long base = (long long)tile * TILE + (long long)w * WARP_CHUNK;
  unsigned int key[ITEMS], val[ITEMS], rank[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    long long idx = base + r * 32 + lane;
    bool valid = idx < n;
    key[r] = valid ? __ldg(keys_in + idx) : 0u;
    val[r] = valid ? __ldg(vals_in + idx) : 0u;
  }
  const unsigned int lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    long long idx = base + r * 32 + lane;
    bool valid = idx < n;
    unsigned int d = valid ? ((key[r] >> shift) & (RADIX - 1)) : (unsigned int)RADIX;
    unsigned int peers = __match_any_sync(0xffffffffu, d);
    unsigned int before = __popc(peers & lt_mask);
    unsigned int b0 = valid ? wcnt[w][d] : 0u;
    __syncwarp();
    if (valid && before == 0) wcnt[w][d] = b0 + __popc(peers);
    __syncwarp();
    rank[r] = b0 + before;
  }
  __syncthreads();
  // per digit: exclusive scan over warps, plus the tile's global offset
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
    unsigned int run = hist_scan[(long long)d * num_tiles + tile];
#pragma unroll
    for (int ww = 0; ww < SORT_WARPS; ++ww) {
      unsigned int c = wcnt[ww][d];
      wcnt[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; ++r) {
    long long idx = base + r * 32 + lane;
    if (idx < n) {
      unsigned int d = (key[r] >> shift) & (RADIX - 1);
      unsigned int pos = wcnt[w][d] + rank[r];
      keys_out[pos] = key[r];
      vals_out[pos] = val[r];
    }
  }
}

// cell_start[c] = first sorted slot whose key >= c, for c in [0, Nc] (Nc = sentinel).
__global__ void k_cell_bounds(const unsigned int *__restrict__ keys, const DevCounters *cnt, unsigned int sentinel,
                              int *__restrict__ cell_start) {
  const int n = cnt->n_sorted;
  long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s > n) return;
  long long prev = (s == 0) ? -1 : (long long)keys[s - 1];
  long long cur = (s == n) ? (long long)sentinel : (long long)keys[s];
  if (cur > (long long)sentinel) cur = sentinel;
  for (long long c = prev + 1; c <= cur; ++c) cell_start[c] = (int)s;
}

__global__ void k_update_counts(DevCounters *cnt, const int *cell_start, unsigned int sentinel, int drop_removed) {
  int live = cell_start[sentinel];
  cnt->n = live;
  if (drop_removed) cnt->n_sorted = live;
}

}  // namespace

size_t radix_scratch_bytes(int n_cap) {
  long long tiles = ((long long)n_cap + TILE - 1) / TILE;
  if (tiles < 1) tiles = 1;
  long long hist = tiles * RADIX;
  long long sums = (hist + SCAN_BLOCK - 1) / SCAN_BLOCK;
  auto al = [](long long b) { return (size_t)((b + 255) / 256 * 256); };
  return al(4LL * n_cap) * 2 + al(4 * hist) + al(4 * (sums + 1));
}

void radix_scratch_carve(void *base, int n_cap, RadixScratch *rs) {
  long long tiles = ((long long)n_cap + TILE - 1) / TILE;
  if (tiles < 1) tiles = 1;
  long long hist = tiles * RADIX;
  auto al = [](long long b) { return (size_t)((b + 255) / 256 * 256); };
  char *p = (char *)base;
  rs->keys_alt = (unsigned int *)p; p += al(4LL * n_cap);
  rs->vals_alt = (unsigned int *)p; p += al(4LL * n_cap);
  rs->hist = (unsigned int *)p; p += al(4 * hist);
  rs->hist_scan_tmp = (unsigned int *)p;
  rs->cap_items = n_cap;
  rs->cap_tiles = (int)tiles;
}

static void exclusive_scan_u32(unsigned int *data, long long count, unsigned int *sums, cudaStream_t s) {
  long long blocks = (count + SCAN_BLOCK - 1) / SCAN_BLOCK;
  k_scan_reduce<<<(unsigned)blocks, SCAN_THREADS, 0, s>>>(data, count, sums);
  k_scan_sums<<<1, SCAN_THREADS, 0, s>>>(sums, (int)blocks);
  k_scan_apply<<<(unsigned)blocks, SCAN_THREADS, 0, s>>>(data, count, sums);
}

void radix_sort_pairs(unsigned int **keys, unsigned int **vals, const int *n_dev, int bits, RadixScratch &rs,
                      cudaStream_t s) {
  int tiles = rs.cap_tiles;
  unsigned int *kin = *keys, *vin = *vals, *kout = rs.keys_alt, *vout = rs.vals_alt;
  int passes = (bits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    int shift = 8 * p;
    k_hist<<<tiles, SORT_THREADS, 0, s>>>(kin, n_dev, shift, rs.hist, tiles);
    exclusive_scan_u32(rs.hist, (long long)tiles * RADIX, rs.hist_scan_tmp, s);
    k_scatter<<<tiles, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, n_dev, shift, rs.hist, tiles);
    unsigned int *tk = kin, *tv = vin;
    kin = kout; vin = vout; kout = tk; vout = tv;
  }
  // the sorted pairs are in (kin, vin); hand the other pair back as scratch
  *keys = kin; *vals = vin;
  rs.keys_alt = kout; rs.vals_alt = vout;
}

void launch_cell_bounds(const unsigned int *keys, int n_cap, const DevCounters *cnt, unsigned int sentinel,
                        int *cell_start, cudaStream_t s) {
  int th = 256;
  long long blocks = ((long long)n_cap + 1 + th - 1) / th;
  k_cell_bounds<<<(unsigned)blocks, th, 0, s>>>(keys, cnt, sentinel, cell_start);
}

void launch_update_counts(DevCounters *cnt, const int *cell_start, unsigned int sentinel, int drop_removed,
                          cudaStream_t s) {
  k_update_counts<<<1, 1, 0, s>>>(cnt, cell_start, sentinel, drop_removed);
}
