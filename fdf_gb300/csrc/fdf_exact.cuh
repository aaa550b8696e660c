// fdf_exact.cuh -- IEEE-exact helpers for the FP64 parity path.
//
// GB300 executes FP64 adds and multiplies at ~1/64 of the FP32 rate, so the
// plain path keeps the FP64 pipe for arithmetic the reference actually rounds
// and moves everything else to the integer pipe.  Every helper here returns
// exactly what the corresponding C expression returns, for all inputs
// (signed zeros, infinities and NaNs included):
//   abs_lt(d, t)  == (fabs(d) < t)
//   lt0(d)        == (d < 0.0)
//   eq0(d)        == (d == 0.0)
//   le(d, c)      == (d <= c)        for a finite positive constant c
//   add0(x)       == (0.0 + x)       (only -0.0 changes: it becomes +0.0)
// The _rn intrinsics are never contracted into an FMA, whatever the flags.
#pragma once
#include <cuda_runtime.h>

namespace fdfx {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }

constexpr unsigned long long ABS_MASK = 0x7fffffffffffffffULL;
constexpr unsigned long long INF_BITS = 0x7ff0000000000000ULL;
constexpr unsigned long long NEG_ZERO = 0x8000000000000000ULL;

__device__ __forceinline__ unsigned long long ubits(double x) { return (unsigned long long)__double_as_longlong(x); }

__device__ __forceinline__ bool is_nan(double x) { return (ubits(x) & ABS_MASK) > INF_BITS; }

// fabs(d) < t.  tb = bits of t; t_nan: t is NaN (then the comparison is false).
__device__ __forceinline__ bool abs_lt_bits(double d, unsigned long long tb, bool t_nan) {
  // t >= 0 here (a threshold); for t = -0.0 or +0.0 nothing is below it.
  return !t_nan && ((ubits(d) & ABS_MASK) < (tb & ABS_MASK)) && !((tb >> 63) && (tb & ABS_MASK));
}

__device__ __forceinline__ bool lt0(double d) {
  unsigned long long b = ubits(d), a = b & ABS_MASK;
  return (b >> 63) && a != 0 && a <= INF_BITS;
}

__device__ __forceinline__ bool eq0(double d) { return (ubits(d) & ABS_MASK) == 0; }

// d <= c for a finite, positive constant c (cb = bits of c).
__device__ __forceinline__ bool le_pos(double d, unsigned long long cb) {
  unsigned long long b = ubits(d), a = b & ABS_MASK;
  if (a > INF_BITS) return false;   // NaN
  if (b >> 63) return true;         // negative or -0.0
  return b <= cb;
}

__device__ __forceinline__ double add0(double x) { return ubits(x) == NEG_ZERO ? 0.0 : x; }

// (double)n for 0 <= n < 2^31, built on the integer pipe (exact: n has < 53 bits).
__device__ __forceinline__ double u32_to_double(unsigned int n) {
  if (n == 0) return 0.0;
  const int e = 31 - __clz((int)n);                              // floor(log2 n)
  const unsigned long long mant = ((unsigned long long)n << (52 - e)) & 0x000fffffffffffffULL;
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | mant));
}

// x / n for an integer count n >= 1: x for n = 1, x * 2^-k (exact) for n = 2^k,
// else the correctly rounded division -- all three equal the IEEE quotient.
__device__ __forceinline__ double div_count(double x, unsigned int n) {
  if (n == 1) return x;
  if ((n & (n - 1)) == 0) {
    const int e = 31 - __clz((int)n);
    return __dmul_rn(x, __longlong_as_double((long long)((unsigned long long)(1023 - e) << 52)));
  }
  return __ddiv_rn(x, u32_to_double(n));
}

// PETSc's PetscMin / PetscMax macros: a<b ? a : b and a<b ? b : a.
__device__ __forceinline__ double pmin(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double pmax(double a, double b) { return (a < b) ? b : a; }

// PetscMax(0.0, PetscMin(1.0, a)) of ComputeTrilinearWeights, on the integer pipe:
// a > 1 -> 1; NaN or a <= 0 (incl. -0.0) -> +0.0; else a.
__device__ __forceinline__ double clamp01(double a) {
  unsigned long long b = ubits(a), m = b & ABS_MASK;
  const unsigned long long ONE = 0x3ff0000000000000ULL;
  if (m > INF_BITS) return 0.0;                 // PetscMin(1, NaN) = NaN; PetscMax(0, NaN) = 0
  if (b >> 63) return 0.0;                      // negative or -0.0: 0.0 < x false -> 0.0
  if (b == 0) return 0.0;
  if (b > ONE) return 1.0;
  return a;
}

}  // namespace fdfx
