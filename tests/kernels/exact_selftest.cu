// Self-test of the off-FP64-pipe helpers in fdf_exact.cuh against the hardware instructions
// they replace, bit for bit: div_rn / div_by against __ddiv_rn, mul_int against __dmul_rn,
// d2f_rn against __double2float_rn, split_rn against (fl32(x), fl32(x - fl32(x))), scale_down
// against the multiply by 2^-k, in_range, lt0, eq0, is_nan, abs_lt_bits, le_pos, add0 and
// clamp01 against the C comparisons and expressions they restate.  Operands come seeded
// from several distributions: random bit patterns with every exponent, the fast range, divisors
// near 1, extreme significands, short significands (whose products hit exact ties), operands a
// few ulps apart with opposite signs, zeros, subnormals, infinities and NaNs.  Test
// infrastructure: built by the GPU tests, not part of the library.
#include <cstdint>
#include <cuda_runtime.h>

#include "fdf_exact.cuh"

namespace {

__device__ __forceinline__ uint64_t mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// An operand from distribution k of 8, from the random word r.
__device__ double operand(uint64_t r, int k) {
  const uint64_t frac = r & 0x000fffffffffffffull, sgn = (r >> 63) << 63;
  const uint64_t e = (r >> 52) & 0x7ffull;
  switch (k) {
    case 0: return __longlong_as_double((long long)r);                                   // any bit pattern
    case 1: return __longlong_as_double((long long)(sgn | ((960ull + (e % 128)) << 52) | frac));   // moderate range
    case 2: return __longlong_as_double((long long)(((1023ull + (e % 3) - 1) << 52) | frac));   // near 1
    case 3: {                                                                            // 1 +- a few ulps
      const long long k2 = (long long)(e % 17) - 8;
      return 1.0 + (double)k2 * 0x1p-52;
    }
    case 4: {                                                                            // extreme significands
      const uint64_t f[4] = {0ull, 1ull, 0x000fffffffffffffull, 0x000ffffffffffffeull};
      return __longlong_as_double((long long)(sgn | ((1000ull + (e % 48)) << 52) | f[(r >> 8) & 3]));
    }
    case 5: return __longlong_as_double((long long)(sgn | ((e % 64) << 52) | frac));   // subnormal / tiny
    case 6: return __longlong_as_double((long long)(sgn | ((1985ull + (e % 63)) << 52) | frac));   // huge, inf, NaN
    default: {                                                                           // a small integer count
      return (double)(1 + (r % 1000));
    }
  }
}

// Keeps the top m bits of the significand (m = 1..53 from r).
__device__ __forceinline__ double shorten(double x, uint64_t r) {
  const int m = 1 + (int)(r % 53);
  const uint64_t keep = ~((1ull << (53 - m)) - 1ull);
  return __longlong_as_double((long long)((uint64_t)__double_as_longlong(x) & (0xfff0000000000000ull | (keep & 0x000fffffffffffffull))));
}

__device__ __forceinline__ bool same(double a, double b) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
  const bool na = (ua & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
  const bool nb = (ub & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
  return (na && nb) || ua == ub;
}
__device__ __forceinline__ bool samef(float a, float b) {
  return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}

// out[0..2]: division, d2f, split mismatches; out[4..5]: the first bad division's operands;
// out[6]: scale_down, out[7]: mul_int, out[8]: in_range, out[9]: bit-predicate mismatches.
__global__ void k_check(uint64_t seed, long long n, unsigned long long *out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const uint64_t r1 = mix(seed ^ (2 * (uint64_t)t)), r2 = mix(seed ^ (2 * (uint64_t)t + 1)), r3 = mix(r1 ^ r2);
    double a = operand(r1, (int)(r3 & 7)), b = operand(r2, (int)((r3 >> 3) & 7));
    if ((r3 >> 20) & 1) a = shorten(a, r3 >> 24);
    if ((r3 >> 21) & 1) b = shorten(b, r3 >> 32);
    if (((r3 >> 22) & 7) == 0) {   // b = -(a +- a few ulps): cancellation
      const long long k = (long long)((r3 >> 40) % 9) - 4;
      b = __longlong_as_double(__double_as_longlong(a) + k) * -1.0;
    }
    const double q = fdfx::div_rn(a, b), qh = __ddiv_rn(a, b);
    if (!same(q, qh)) {
      if (atomicAdd(&out[0], 1ull) == 0ull) {
        out[4] = (unsigned long long)__double_as_longlong(a);
        out[5] = (unsigned long long)__double_as_longlong(b);
      }
    }
    if (!samef(fdfx::d2f_rn(a), __double2float_rn(a))) atomicAdd(&out[1], 1ull);
    const float2 p = fdfx::split_rn(a);
    const float h = __double2float_rn(a);
    const float l = __double2float_rn(__dsub_rn(a, (double)h));
    if (!samef(p.x, h) || !samef(p.y, l)) atomicAdd(&out[2], 1ull);
    if (!same(fdfx::mul_int(a, b), __dmul_rn(a, b))) atomicAdd(&out[7], 1ull);
    {   // in_range against the FP64 comparisons, with a third operand from the same distributions
      const double c = operand(r3 ^ r1, (int)((r3 >> 48) & 7));
      const double lo = ((r3 >> 51) & 1) ? b : c, hi = ((r3 >> 51) & 1) ? c : b;
      if (fdfx::in_range(a, lo, hi) != (a >= lo && a <= hi)) atomicAdd(&out[8], 1ull);
    }
    {   // the predicates on the bits against the C comparisons they restate
      const double t = fabs(b);
      bool bad = fdfx::lt0(a) != (a < 0.0) || fdfx::eq0(a) != (a == 0.0) || fdfx::is_nan(a) != (a != a);
      bad = bad || fdfx::abs_lt_bits(a, fdfx::ubits(t), t != t) != (fabs(a) < t);
      if (t == t && t > 0.0 && t < 1.0e300) bad = bad || fdfx::le_pos(a, fdfx::ubits(t)) != (a <= t);
      bad = bad || !same(fdfx::add0(a), 0.0 + a);
      const double m1 = (1.0 < a) ? 1.0 : a;        // PetscMin(1.0, a) = 1.0 < a ? 1.0 : a
      const double cl = (0.0 < m1) ? m1 : 0.0;      // PetscMax(0.0, m1) = 0.0 < m1 ? m1 : 0.0
      bad = bad || !same(fdfx::clamp01(a), cl);
      if (bad) atomicAdd(&out[9], 1ull);
    }
    const int k = (int)((r3 >> 8) % 53);
    if (!same(fdfx::scale_down(a, k), __dmul_rn(a, __longlong_as_double((long long)((uint64_t)(1023 - k) << 52)))))
      atomicAdd(&out[6], 1ull);
  }
}

}  // namespace

// Runs n cases from the seed; writes the ten counters to host memory.  Returns a CUDA error code.
extern "C" int fdf_test_exact(unsigned long long seed, long long n, unsigned long long *host_out) {
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMalloc((void **)&d, 10 * sizeof(unsigned long long));
  if (e != cudaSuccess) return (int)e;
  e = cudaMemset(d, 0, 10 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    k_check<<<152 * 8, 256>>>(seed, n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host_out, d, 10 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  host_out[3] = (unsigned long long)n;
  return (int)e;
}
