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

constexpr unsigned long long ABS_MASK = 0x7fffffffffffffffULL;
constexpr unsigned long long INF_BITS = 0x7ff0000000000000ULL;
constexpr unsigned long long NEG_ZERO = 0x8000000000000000ULL;

// The bits of x through a move the compiler cannot see into: a plain reinterpretation lets it
// fold the integer tests below (x == 0 through the magnitude bits, NaN through the exponent,
// range tests) back into FP64 comparisons, which then run on the FP64 pipe this path is bound
// by (measured: 9 to 18 such instructions per particle in the plain kernels).
__device__ __forceinline__ unsigned long long ubits(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}

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

// A signed integer with the order of the doubles (both zeros map to 0); for non-NaN values,
// x <= y exactly when key(x) <= key(y).
__device__ __forceinline__ long long order_key(double x) {
  const unsigned long long b = ubits(x);
  return (b >> 63) ? -(long long)(b & ABS_MASK) : (long long)b;
}

// x >= lo && x <= hi, on the integer pipe (false when any of the three is NaN).
__device__ __forceinline__ bool in_range(double x, double lo, double hi) {
  const long long k = order_key(x);
  return !is_nan(x) && !is_nan(lo) && !is_nan(hi) && k >= order_key(lo) && k <= order_key(hi);
}

// (double)n for 0 <= n < 2^31, built on the integer pipe (exact: n has < 53 bits).
__device__ __forceinline__ double u32_to_double(unsigned int n) {
  if (n == 0) return 0.0;
  const int e = 31 - __clz((int)n);                              // floor(log2 n)
  const unsigned long long mant = ((unsigned long long)n << (52 - e)) & 0x000fffffffffffffULL;
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | mant));
}

// ---------------------------------------------------------------------------------------
// Division and conversions off the FP64 pipe.  On GB300 one warp-wide FP64 instruction holds
// an SM sub-partition's FP64 unit for 64 cycles, while FP32 and integer instructions issue
// every cycle or two; a correctly rounded double division (about ten FP64 instructions) or a
// double <-> float conversion therefore costs far more than the same result built from
// integer and FP32 operations.  Each routine below returns the IEEE result bit for bit; inputs
// outside its fast range go to the hardware instruction, kept out of line so that the
// compiler does not if-convert it into every lane.

static __device__ __noinline__ double div_hw(double a, double b) { return __ddiv_rn(a, b); }
static __device__ __noinline__ float d2f_hw(double x) { return __double2float_rn(x); }

// double -> float, round to nearest even, on the integer pipe for results in the normal
// float range; the rest takes the hardware conversion.  The low 29 mantissa bits round into
// bit 29 (ties to even), a carry moves into the exponent, and the exponent is rebased from
// 1023 to 127.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long b = ubits(x);
  const unsigned long long mag = b & ABS_MASK;
  if (mag >= 0x3810000000000000ull && mag < 0x47efffffe0000000ull) {   // [2^-126, FLT_MAX)
    const unsigned long long r = mag + 0x0fffffffull + ((mag >> 29) & 1ull);
    const unsigned int f = (unsigned int)(r >> 29) - ((1023u - 127u) << 23);
    return __uint_as_float(f | ((unsigned int)(b >> 32) & 0x80000000u));
  }
  return d2f_hw(x);
}

static __device__ __noinline__ float2 split_hw(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(__dsub_rn(x, (double)h)));
}

// (hi, lo) = (fl32(x), fl32(x - fl32(x))): |x - (hi + lo)| <= 2^-48 |x|.  For 2^-74 <= |x| <
// 2^127 it is built on the integer and FP32 pipes: hi as in d2f_rn; x - hi is an integer
// number of x's ulps (|.| <= 2^28, the difference of the two bit patterns, which stays exact
// across a binade carry), converted to float (one rounding: fl32(x - hi)) and scaled by
// ulp(x) = 2^(E - 1075), a normal float there.  Zero gives (x, 0); the rest goes through FP64.
__device__ __forceinline__ float2 split_rn(double x) {
  const unsigned long long b = ubits(x);
  const unsigned long long mag = b & ABS_MASK;
  const unsigned int sgn = (unsigned int)(b >> 32) & 0x80000000u;
  if (mag >= 0x3b50000000000000ull && mag < 0x47e0000000000000ull) {
    const unsigned long long r = mag + 0x0fffffffull + ((mag >> 29) & 1ull);
    const unsigned long long hmag = r & ~0x1fffffffull;
    const float hi = __uint_as_float(((unsigned int)(r >> 29) - ((1023u - 127u) << 23)) | sgn);
    const int units = (int)((long long)mag - (long long)hmag);
    const float ulp = __uint_as_float((unsigned int)((mag >> 52) - 948ull) << 23);
    const float lo = __fmul_rn(__int2float_rn(units), ulp);                 // x - hi == 0 gives +0
    return make_float2(hi, __uint_as_float(__float_as_uint(lo) ^ (units != 0 ? sgn : 0u)));
  }
  if (mag == 0ull) return make_float2(__uint_as_float(sgn), 0.0f);
  return split_hw(x);
}

// Correctly rounded a / b (round to nearest even) from integer and FP32 operations, for
// normal a (or zero) and b with a normal quotient; other operands take the hardware divide.
// With ma, mb the 53-bit significands and s = 53 (ma >= mb) or 54, the quotient's 54-bit
// truncation is Q = floor(ma 2^s / mb) and the result's significand is (Q + 1) >> 1: an exact
// tie would need ma 2^s = mb Q with Q odd, impossible since mb < 2^53 cannot hold the factor
// 2^s, so the rounding bit alone decides.  Q is found in three steps:
//   1. a double-float quotient from 24 + 23-bit parts of ma and mb and a Newton-refined FP32
//      reciprocal, |Q1 - Q| < 2^11;
//   2. the exact remainder R1 = ma 2^s - Q1 mb (128-bit; |R1| < 2^65), its top bits times the
//      reciprocal give the integer correction dl with |R1 / mb - dl| < 0.51;
//   3. R2 = R1 - dl mb (exact in 64 bits), and Q = Q1 + dl - (R2 < 0).
// A divisor used several times is prepared once (Divisor).
struct Divisor {
  double b;
  unsigned long long ub, mb;
  float fbh, fbl, r;
  int eb;
  bool normal;
};

__device__ __forceinline__ Divisor make_divisor(double b) {
  Divisor d;
  d.b = b;
  d.ub = ubits(b);
  d.eb = (int)((d.ub >> 52) & 0x7ff);
  d.normal = d.eb != 0 && d.eb != 0x7ff;
  d.mb = (d.ub & 0x000fffffffffffffull) | 0x0010000000000000ull;
  d.fbh = __uint_as_float(0x3f800000u | ((unsigned int)(d.mb >> 29) & 0x7fffffu));   // bits 52..29, in [1, 2)
  d.fbl = __fmul_rn(__fsub_rn(__uint_as_float(0x4b000000u | ((unsigned int)(d.mb >> 6) & 0x7fffffu)), 8388608.0f),
                    0x1p-46f);                                                       // bits 28..6
  const float r0 = __fdividef(1.0f, d.fbh);                 // within 2 ulps
  d.r = __fmaf_rn(r0, __fmaf_rn(-d.fbh, r0, 1.0f), r0);     // one Newton step
  return d;
}

__device__ __forceinline__ double div_by(double a, const Divisor &d) {
  const unsigned long long ua = ubits(a);
  const unsigned long long sign = (ua ^ d.ub) & NEG_ZERO;
  const int ea = (int)((ua >> 52) & 0x7ff), de = ea - d.eb;
  if ((ua & ABS_MASK) == 0ull && d.normal) return __longlong_as_double((long long)sign);
  if (!d.normal || ea == 0 || ea == 0x7ff || de < -1021 || de > 1021) return div_hw(a, d.b);
  const unsigned long long ma = (ua & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const float fah = __uint_as_float(0x3f800000u | ((unsigned int)(ma >> 29) & 0x7fffffu));
  const float fal = __fmul_rn(__fsub_rn(__uint_as_float(0x4b000000u | ((unsigned int)(ma >> 6) & 0x7fffffu)), 8388608.0f),
                              0x1p-46f);
  const float qh = __fmul_rn(fah, d.r);
  const float p = __fmul_rn(qh, d.fbh);
  const float pe = __fmaf_rn(qh, d.fbh, -p);                              // exact error of p
  const float rem = __fadd_rn(__fsub_rn(__fsub_rn(fah, p), pe), __fmaf_rn(-qh, d.fbl, fal));
  const float ql = __fmul_rn(rem, d.r);
  const int ge = ma >= d.mb;
  const int s = 54 - ge;
  const unsigned int qb = __float_as_uint(qh);
  const int sh = s - 23 + (int)((qb >> 23) & 0xffu) - 127;              // qh in (0.5, 2): 29..32
  unsigned long long Q = ((unsigned long long)((qb & 0x7fffffu) | 0x800000u) << sh) +
                         (unsigned long long)((long long)__float2int_rn(__fmul_rn(ql, ge ? 0x1p42f : 0x1p43f)) << 11);
  // R1 = ma 2^s - Q mb as (R_hi, R_lo), two's complement
  const unsigned long long n_lo = ma << s, n_hi = ma >> (64 - s);
  const unsigned long long p_lo = Q * d.mb, p_hi = __umul64hi(Q, d.mb);
  const unsigned long long r_lo = n_lo - p_lo;
  const unsigned long long r_hi = n_hi - p_hi - (n_lo < p_lo ? 1ull : 0ull);
  const int t = (int)(unsigned int)((r_hi << 29) | (r_lo >> 35));          // R1 >> 35
  const int dl = __float2int_rn(__fmul_rn(__fmul_rn(__int2float_rn(t), d.r), 0x1p-17f));
  Q += (unsigned long long)(long long)dl;
  const long long r2 = (long long)(r_lo - (unsigned long long)((long long)dl * (long long)d.mb));
  Q -= (r2 < 0) ? 1ull : 0ull;
  const unsigned long long qr = (Q + 1ull) >> 1;                           // [2^52, 2^53]
  const unsigned long long e1 = (unsigned long long)(de + 1021 + ge);      // biased exponent - 1
  return __longlong_as_double((long long)(sign | ((e1 << 52) + qr)));
}

__device__ __forceinline__ double div_rn(double a, double b) { return div_by(a, make_divisor(b)); }

// x * 2^-k for 0 <= k <= 52: an exponent decrement on the integer pipe while the product stays
// normal (then exact, as the FP64 multiply is); zeros, infinities and NaNs are their own
// products; a subnormal product takes the FP64 multiply, which rounds it.
static __device__ __noinline__ double mul_hw(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double scale_down(double x, int k) {
  const unsigned long long b = ubits(x);
  const unsigned long long e = (b >> 52) & 0x7ffull;
  if (e > (unsigned long long)k && e != 0x7ffull) return __longlong_as_double((long long)(b - ((unsigned long long)k << 52)));
  if ((b & ABS_MASK) == 0ull || e == 0x7ffull) return x;
  return mul_hw(x, __longlong_as_double((long long)((unsigned long long)(1023 - k) << 52)));
}

// a * b, round to nearest even, on the integer pipe: the same bits as __dmul_rn.  GB300 issues
// FP64 at 1/64 of the FP32 rate while the integer pipe idles in the FP64-bound kernels, so
// routing part of a kernel's FP64 operations here runs both pipes at once.  Fast path: normal
// or zero operands with a normal product; the rest takes the hardware multiply out of line.
constexpr unsigned long long FRAC_MASK = 0x000fffffffffffffull, HIDDEN = 0x0010000000000000ull;

// The 53 x 53-bit significand product P in [2^104, 2^106) is exact in 128 bits; its top 53 bits
// (from bit 52 or 53) are the significand, the bits below decide the rounding (ties to even).
__device__ __forceinline__ double mul_int(double a, double b) {
  const unsigned long long ua = ubits(a), ub = ubits(b);
  const unsigned long long sign = (ua ^ ub) & NEG_ZERO;
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  const int e = ea + eb - 1023;   // biased exponent for a significand product in [1, 2)
  if (ea == 0 || eb == 0 || ea == 0x7ff || eb == 0x7ff || e < 1 || e > 2044) {
    if (((ua & ABS_MASK) == 0ull && eb != 0x7ff) || ((ub & ABS_MASK) == 0ull && ea != 0x7ff))
      return __longlong_as_double((long long)sign);   // zero times a finite value
    return mul_hw(a, b);
  }
  const unsigned long long ma = (ua & FRAC_MASK) | HIDDEN, mb = (ub & FRAC_MASK) | HIDDEN;
  const unsigned long long lo = ma * mb, hi = __umul64hi(ma, mb);
  const unsigned int top = (unsigned int)(hi >> 41) & 1u;   // P >= 2^105
  const int sh = 52 + (int)top;
  const unsigned long long mant = (hi << (64 - sh)) | (lo >> sh);
  const unsigned long long rem = lo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  const unsigned long long up = (rem > half || (rem == half && (mant & 1ull))) ? 1ull : 0ull;
  return __longlong_as_double((long long)(sign | (((unsigned long long)(e - 1 + (int)top) << 52) + mant + up)));
}

// x / n for an integer count n >= 1: x for n = 1, x * 2^-k (exact) for n = 2^k,
// else the correctly rounded division -- all three equal the IEEE quotient.
__device__ __forceinline__ double div_count(double x, unsigned int n) {
  if (n == 1) return x;
  if ((n & (n - 1)) == 0) return scale_down(x, 31 - __clz((int)n));
  return div_rn(x, u32_to_double(n));
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
