// fdf_sort.cu -- per-step re-sort of the particles by cell (a counting sort).
//
//   1. the locate kernel histograms the new cell keys (count[c], integer atomics,
//      warp-aggregated: exact and order-independent);
//   2. an exclusive scan turns count[0..Nc+1) into cell_start[0..Nc+1]: cell c
//      owns sorted slots [cell_start[c], cell_start[c+1]); bucket Nc holds the LOST
//      particles the initial setup keeps, and removed particles get no slot;
//   3. each particle takes slot cell_start[key] + its rank within its cell, which the
//      histogram atomic of step 1 returned;
//   4. each cell's slots are then ordered by (PID, previous slot) in the plain form, so
//      the final order -- and every later sum -- is the same on every run, whatever
//      order the atomics took, and does not depend on the history of the swarm: sorted
//      order is (cell, PID), the order the oracle uses for the face deposits, which makes
//      those sums comparable bit for bit.  The precision forms order each cell's slots by
//      previous slot alone (a stable counting sort: the same on every run for the same
//      input, and no gather of the PIDs), as does the standalone sort.
#include "fdf_internal.cuh"

namespace {

// ---- exclusive scan of a u32 array (reduce -> scan of block sums -> scan with offsets) ----
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_BLOCK = SCAN_THREADS * SCAN_ITEMS;   // 8192 values per block
constexpr int SUMS_PER_THREAD = 16;                      // up to 16384 blocks -> 134M values

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

// Loads SCAN_ITEMS (= 8) consecutive values as two 16-B vectors when the block is
// fully inside and the base is aligned, element by element otherwise.
__device__ __forceinline__ void load8(const unsigned int *__restrict__ in, long long base, long long count,
                                      unsigned int v[SCAN_ITEMS]) {
  if (base + SCAN_ITEMS <= count && ((reinterpret_cast<size_t>(in + base) & 15) == 0)) {
    const uint4 a = *reinterpret_cast<const uint4 *>(in + base);
    const uint4 b = *reinterpret_cast<const uint4 *>(in + base + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; ++q) v[q] = (base + q < count) ? in[base + q] : 0u;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const unsigned int *__restrict__ in, long long count,
                                                             unsigned int *__restrict__ sums) {
  long long base = (long long)blockIdx.x * SCAN_BLOCK + (long long)threadIdx.x * SCAN_ITEMS;
  unsigned int v[SCAN_ITEMS], t = 0;
  load8(in, base, count, v);
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q) t += v[q];
  unsigned int tot;
  block_exclusive_scan(t, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(unsigned int *sums, int nsums) {
  int base = threadIdx.x * SUMS_PER_THREAD;
  unsigned int v[SUMS_PER_THREAD], t = 0;
#pragma unroll
  for (int q = 0; q < SUMS_PER_THREAD; ++q) { v[q] = (base + q < nsums) ? sums[base + q] : 0u; t += v[q]; }
  unsigned int ex = block_exclusive_scan(t, nullptr);
#pragma unroll
  for (int q = 0; q < SUMS_PER_THREAD; ++q) {
    if (base + q < nsums) sums[base + q] = ex;
    ex += v[q];
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(unsigned int *__restrict__ data, long long count,
                                                            const unsigned int *__restrict__ sums) {
  long long base = (long long)blockIdx.x * SCAN_BLOCK + (long long)threadIdx.x * SCAN_ITEMS;
  unsigned int v[SCAN_ITEMS], t = 0;
  load8(data, base, count, v);
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q) t += v[q];
  unsigned int ex = block_exclusive_scan(t, nullptr) + sums[blockIdx.x];
  unsigned int o[SCAN_ITEMS];
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; ++q) { o[q] = ex; ex += v[q]; }
  if (base + SCAN_ITEMS <= count && ((reinterpret_cast<size_t>(data + base) & 15) == 0)) {
    *reinterpret_cast<uint4 *>(data + base) = make_uint4(o[0], o[1], o[2], o[3]);
    *reinterpret_cast<uint4 *>(data + base + 4) = make_uint4(o[4], o[5], o[6], o[7]);
  } else {
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; ++q)
      if (base + q < count) data[base + q] = o[q];
  }
}

// Slot of every kept particle: cell_start[key] + its rank among the particles of the same
// key, which the locate kernels took from their histogram atomics.  Each thread handles
// FDF_SCATTER_ITEMS particles (strided by the block, so every load stays coalesced) and issues
// all their loads before their stores: the cell_start gather depends on the key, so a thread
// with one particle waits two load latencies for one store (sort stage per 64M-particle step:
// 0.78 ms with one particle per thread, 0.66 with 2, 0.61 with 4, 0.63 with 8).
#ifndef FDF_SCATTER_ITEMS
#define FDF_SCATTER_ITEMS 4
#endif
__global__ void __launch_bounds__(256) k_scatter_slots(const unsigned int *__restrict__ keys,
                                                      const unsigned int *__restrict__ rank, const DevCounters *cnt,
                                                      unsigned int sentinel, int keep_lost,
                                                      const unsigned int *__restrict__ cell_start,
                                                      unsigned int *__restrict__ perm) {
  constexpr int IT = FDF_SCATTER_ITEMS;
  const long long n = cnt->n_sorted;
  const long long base = (long long)blockIdx.x * IT * blockDim.x + threadIdx.x;
  unsigned int key[IT], start[IT], rk[IT];
  bool keep[IT];
#pragma unroll
  for (int q = 0; q < IT; ++q) {
    const long long s = base + (long long)q * blockDim.x;
    key[q] = s < n ? keys[s] : 0xffffffffu;   // sentinel: a LOST particle kept at the end; above: removed
    keep[q] = key[q] < sentinel || (key[q] == sentinel && keep_lost);
  }
#pragma unroll
  for (int q = 0; q < IT; ++q) {
    const long long s = base + (long long)q * blockDim.x;
    start[q] = keep[q] ? cell_start[key[q]] : 0u;
    rk[q] = keep[q] ? rank[s] : 0u;
  }
#pragma unroll
  for (int q = 0; q < IT; ++q)
    if (keep[q]) perm[start[q] + rk[q]] = (unsigned int)(base + (long long)q * blockDim.x);
}

// Orders every cell's slots by (PID, previous slot) -- or by previous slot alone when
// pid is null.  Segments are short (a few particles per cell on average): up to 8 entries
// are checked and, when out of order, sorted in registers by a 19-comparator sorting
// network; longer ones are insertion-sorted in place in global memory.
constexpr int SEG_NET = 8;

__device__ __forceinline__ bool key_gt(long long ka, unsigned int va, long long kb, unsigned int vb) {
  return ka > kb || (ka == kb && va > vb);
}

// One cell's slots [s0, s0 + L) ordered by (key, previous slot), key = PID or, with pid null,
// the previous slot itself.
__device__ __forceinline__ void order_cell(unsigned int s0, unsigned int L, const long long *__restrict__ pid,
                                           unsigned int *__restrict__ perm) {
  if (L < 2) return;
  if (L <= SEG_NET) {
    long long kp[SEG_NET];
    unsigned int ix[SEG_NET];
    bool sorted = true;
#pragma unroll
    for (int q = 0; q < SEG_NET; ++q) {
      // padding (max, max) sorts after every real entry (slots are below 2^31)
      kp[q] = 0x7fffffffffffffffLL;
      ix[q] = 0xffffffffu;
      if (q < (int)L) {
        ix[q] = perm[s0 + q];
        kp[q] = pid ? pid[ix[q]] : (long long)ix[q];
        if (q > 0 && key_gt(kp[q - 1], ix[q - 1], kp[q], ix[q])) sorted = false;
      }
    }
    if (sorted) return;
    auto cx = [&](int a, int b) {
      const bool sw = key_gt(kp[a], ix[a], kp[b], ix[b]);
      const long long ka = sw ? kp[b] : kp[a], kb = sw ? kp[a] : kp[b];
      const unsigned int va = sw ? ix[b] : ix[a], vb = sw ? ix[a] : ix[b];
      kp[a] = ka; kp[b] = kb; ix[a] = va; ix[b] = vb;
    };
    cx(0, 2); cx(1, 3); cx(4, 6); cx(5, 7);
    cx(0, 4); cx(1, 5); cx(2, 6); cx(3, 7);
    cx(0, 1); cx(2, 3); cx(4, 5); cx(6, 7);
    cx(2, 4); cx(3, 5);
    cx(1, 4); cx(3, 6);
    cx(1, 2); cx(3, 4); cx(5, 6);
#pragma unroll
    for (int q = 0; q < SEG_NET; ++q)
      if (q < (int)L) perm[s0 + q] = ix[q];
  } else {
    for (unsigned int q = 1; q < L; ++q) {
      unsigned int v = perm[s0 + q];
      long long kv = pid ? pid[v] : (long long)v;
      unsigned int r = q;
      while (r > 0) {
        unsigned int u = perm[s0 + r - 1];
        long long ku = pid ? pid[u] : (long long)u;
        if (ku < kv || (ku == kv && u < v)) break;
        perm[s0 + r] = u;
        --r;
      }
      perm[s0 + r] = v;
    }
  }
}

__global__ void __launch_bounds__(256, FDF_ORDER_MIN_BLOCKS) k_order_segments(const unsigned int *__restrict__ cell_start, int nseg,
                                                       const long long *__restrict__ pid,
                                                       unsigned int *__restrict__ perm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nseg) return;
  const unsigned int s0 = cell_start[c];
  order_cell(s0, cell_start[c + 1] - s0, pid, perm);
}

// The order by previous slot (the precision forms and the standalone sort): the keys are the
// slots themselves, so the sorting network compares one 32-bit word per entry (sort stage per
// 64M-particle step 0.61 -> 0.47 ms against the general kernel with a null PID array; two or four
// cells per thread, their loads issued first, measured no faster).
__global__ void __launch_bounds__(256, FDF_ORDER_MIN_BLOCKS) k_order_segments_slot(
    const unsigned int *__restrict__ cell_start, int nseg, unsigned int *__restrict__ perm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nseg) return;
  const unsigned int s0 = cell_start[c], L = cell_start[c + 1] - s0;
  if (L < 2) return;
  if (L > (unsigned int)SEG_NET) {
    order_cell(s0, L, nullptr, perm);
    return;
  }
  unsigned int ix[SEG_NET];
  bool sorted = true;
#pragma unroll
  for (int e = 0; e < SEG_NET; ++e) {   // padding (max) sorts after every slot (slots are below 2^31)
    ix[e] = e < (int)L ? perm[s0 + e] : 0xffffffffu;
    if (e > 0 && e < (int)L && ix[e - 1] > ix[e]) sorted = false;
  }
  if (sorted) return;
  auto cx = [&](int a, int b) {
    const unsigned int va = min(ix[a], ix[b]), vb = max(ix[a], ix[b]);
    ix[a] = va; ix[b] = vb;
  };
  cx(0, 2); cx(1, 3); cx(4, 6); cx(5, 7);
  cx(0, 4); cx(1, 5); cx(2, 6); cx(3, 7);
  cx(0, 1); cx(2, 3); cx(4, 5); cx(6, 7);
  cx(2, 4); cx(3, 5);
  cx(1, 4); cx(3, 6);
  cx(1, 2); cx(3, 4); cx(5, 6);
#pragma unroll
  for (int e = 0; e < SEG_NET; ++e)
    if (e < (int)L) perm[s0 + e] = ix[e];
}

// count[cell[s]] += 1 for 0 <= cell[s] < ncells (warp-aggregated integer atomics)
__global__ void __launch_bounds__(256) k_cell_histogram(const int *__restrict__ cell, long long n, long long ncells,
                                                       unsigned int *__restrict__ count) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned int key = 0xffffffffu;
  if (s < n) {
    const int c = cell[s];
    if (c >= 0 && (long long)c < ncells) key = (unsigned int)c;
  }
  const unsigned int peers = __match_any_sync(0xffffffffu, key);
  if (key != 0xffffffffu && (int)(threadIdx.x & 31) == __ffs(peers) - 1)
    atomicAdd(count + key, (unsigned int)__popc(peers));
}

// slot of every particle with a valid cell (warp-aggregated cursors)
__global__ void __launch_bounds__(256) k_cell_slots(const int *__restrict__ cell, long long n, long long ncells,
                                                   const unsigned int *__restrict__ cell_start,
                                                   unsigned int *__restrict__ cursor, unsigned int *__restrict__ perm) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned int key = 0xffffffffu;
  if (s < n) {
    const int c = cell[s];
    if (c >= 0 && (long long)c < ncells) key = (unsigned int)c;
  }
  const unsigned int peers = __match_any_sync(0xffffffffu, key);
  if (key == 0xffffffffu) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  const unsigned int rank = __popc(peers & ((1u << lane) - 1u));
  unsigned int base = 0;
  if (lane == leader) base = atomicAdd(cursor + key, (unsigned int)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  perm[cell_start[key] + base + rank] = (unsigned int)s;
}

}  // namespace

size_t scan_scratch_words(long long count) { return (size_t)((count + SCAN_BLOCK - 1) / SCAN_BLOCK) + 1; }

long long scan_max_count() { return (long long)SCAN_BLOCK * SCAN_THREADS * SUMS_PER_THREAD; }

void exclusive_scan_u32(unsigned int *data, long long count, unsigned int *sums, cudaStream_t s) {
  long long blocks = (count + SCAN_BLOCK - 1) / SCAN_BLOCK;
  if (blocks < 1) blocks = 1;
  k_scan_reduce<<<(unsigned)blocks, SCAN_THREADS, 0, s>>>(data, count, sums);
  k_scan_sums<<<1, SCAN_THREADS, 0, s>>>(sums, (int)blocks);
  k_scan_apply<<<(unsigned)blocks, SCAN_THREADS, 0, s>>>(data, count, sums);
}

void launch_scatter_slots(const unsigned int *keys, const unsigned int *rank, int n_cap, const DevCounters *cnt,
                          unsigned int sentinel, int keep_lost, const unsigned int *cell_start, unsigned int *perm,
                          cudaStream_t s) {
  const int th = 256, per_block = th * FDF_SCATTER_ITEMS;
  int blocks = (n_cap + per_block - 1) / per_block;
  if (blocks == 0) blocks = 1;
  k_scatter_slots<<<blocks, th, 0, s>>>(keys, rank, cnt, sentinel, keep_lost, cell_start, perm);
}

void launch_order_segments(const unsigned int *cell_start, int nseg, const long long *pid, unsigned int *perm,
                           cudaStream_t s) {
  const int th = 256;
  if (pid) {
    const int blocks = (nseg + th - 1) / th;
    k_order_segments<<<blocks, th, 0, s>>>(cell_start, nseg, pid, perm);
  } else {
    const int blocks = (nseg + th - 1) / th;
    k_order_segments_slot<<<blocks, th, 0, s>>>(cell_start, nseg, perm);
  }
}

// Stable counting sort of particle slots by cell id, on caller-provided scratch:
// cursor [ncells] and sums [scan_scratch_words(ncells + 1)].  cell_start [ncells + 1]
// is both the histogram and (after the scan) the output.
void cell_sort_on_scratch(const int *cell, long long n, long long ncells, unsigned int *perm,
                          unsigned int *cell_start, unsigned int *cursor, unsigned int *sums, cudaStream_t s) {
  cudaMemsetAsync(cell_start, 0, 4ull * (ncells + 1), s);
  cudaMemsetAsync(cursor, 0, 4ull * ncells, s);
  const int th = 256;
  const unsigned int blocks = (unsigned int)((n + th - 1) / th > 0 ? (n + th - 1) / th : 1);
  k_cell_histogram<<<blocks, th, 0, s>>>(cell, n, ncells, cell_start);
  exclusive_scan_u32(cell_start, ncells + 1, sums, s);
  k_cell_slots<<<blocks, th, 0, s>>>(cell, n, ncells, cell_start, cursor, perm);
  launch_order_segments(cell_start, (int)ncells, nullptr, perm, s);
}
