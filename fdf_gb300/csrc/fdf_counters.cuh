// fdf_counters.cuh -- per-step counters of the locate kernels, reduced per block before
// they reach the DevCounters words in global memory: every warp of every block adding to
// the same few addresses serialises in one L2 slice, so each block issues at most one
// atomic per counter.
#pragma once
#include "fdf_internal.cuh"

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Per-thread counts stay far below 2^32 within one launch; the block sums are 64-bit.
struct LocCounts {
  unsigned int lost = 0, oob = 0, evals = 0, done = 0, lost_total = 0, fb = 0;
  unsigned int err = 0;
};

// Histogram of the kept keys: one atomic per distinct key in the warp (all 32 lanes call it;
// hkey = all ones for none).
__device__ __forceinline__ void warp_histogram(unsigned int hkey, unsigned int *__restrict__ count) {
  const unsigned int peers = __match_any_sync(0xffffffffu, hkey);
  const int lane = threadIdx.x & 31;
  if (hkey != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(count + hkey, (unsigned int)__popc(peers));
}

// The same histogram, returning each particle's rank among the particles of its key: a warp's
// particles of one key take consecutive ranks after the count the key had (the atomic's old
// value).  The rank is undefined for hkey = all ones.
__device__ __forceinline__ unsigned int warp_histogram_rank(unsigned int hkey, unsigned int *__restrict__ count) {
  const unsigned int peers = __match_any_sync(0xffffffffu, hkey);
  const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  unsigned int base = 0u;
  if (hkey != 0xffffffffu && lane == leader) base = atomicAdd(count + hkey, (unsigned int)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + (unsigned int)__popc(peers & ((1u << lane) - 1u));
}

// Adds the block's counters to cnt.  Every thread of the block calls it (blockDim.x a
// multiple of 32, at most 1024).
__device__ __forceinline__ void block_flush_counts(const LocCounts &m, DevCounters *cnt) {
  __shared__ unsigned long long red[32][6];
  __shared__ unsigned int rerr[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();   // a previous call's readers are done with the shared words
  unsigned long long v[6] = {m.lost, m.oob, m.evals, m.done, m.lost_total, m.fb};   // widened before the sums
#pragma unroll
  for (int q = 0; q < 6; ++q) v[q] = warp_sum_u64(v[q]);
  const unsigned int e = __reduce_or_sync(0xffffffffu, m.err);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 6; ++q) red[w][q] = v[q];
    rerr[w] = e;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    const int q = threadIdx.x;
    if (q < 6) {
      unsigned long long t = 0;
      for (int k = 0; k < nw; ++k) t += red[k][q];
      // slot q of this block's flush row (CNT_LOST .. CNT_FB are 0 .. 5, the order of v[])
      if (t) atomicAdd(&cnt->stripes[blockIdx.x & (FDF_CNT_STRIPES - 1)][q], t);
    } else {
      unsigned int t = 0;
      for (int k = 0; k < nw; ++k) t |= rerr[k];
      if (t) atomicOr(&cnt->err, t);
    }
  }
}

// Sum of a per-thread count over the block, added to *dst by one thread.  Every thread
// of the block calls it.
__device__ __forceinline__ void block_add_u64(unsigned long long v, unsigned long long *dst) {
  __shared__ unsigned long long part[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();   // a previous call's reader is done with the shared words
  v = warp_sum_u64(v);
  if (lane == 0) part[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int k = 0; k < nw; ++k) t += part[k];
    if (t) atomicAdd(dst, t);
  }
}
