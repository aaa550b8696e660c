// fdf_walk.cuh -- the walking search's cell evaluation with exact decisions from the FP32
// plane table, shared by the plain FP64 walk (fdf_walk.cu) and the precision forms
// (fdf_fp32.cu).  EvaluateParticlePosition / DeterminePointPosition (walkingsearch.c:407-462,
// 811-859) and the index update of UpdateCellIndicesBasedOnDistancesTEST (:882-959).
//
// Each face class the walk needs -- d < 0, d == 0 (|d| < thr), d > 0 -- is decided from an
// FP32 signed distance when that is provably the FP64 class for the position, and from the
// exact FP64 distance (the FP64 plane table, the reference's arithmetic) otherwise.
//
// FP32 distance.  With c0 = c0h + c0l the cell's first vertex as a float pair (exact),
// P = p - c0, E = n . (fc - c0) and d = (fc - p) . n = E - n . P, the row holds n32 = fl32(n)
// and e32 = fl32(E64) (E64: E in FP64), and the kernel computes
//     pr_i = fl32(fl32(ph_i - c0h_i) + fl32(pl_i - c0l_i)),  d32 = e32 - (n32 . pr)
// (the dot product as an FMA chain, then one subtraction).  With B_i = |P_i|,
// ex_i = u (|ph_i| + |c0h_i|), u = 2^-24, eps = 2^-53 and A_i = |fc_i - c0_i|, the roundings
// are bounded by
//     |pr_i - P_i| <= 2u B_i + 2u ex_i                     (the pair subtraction)
//     |e32 - E| <= u |E| + 6 eps sum_i A_i |n_i|            (E64, then fl32)
//     dot product 3u, n32 u, the final subtraction u |d|, the reference's own d64 within
//     5 eps sum_i (A_i + B_i) |n_i| of d,
// which add up to
//     |d32 - d64| <= u S (1 + 12u) + 23 eps sigma,   S = 2 |e32| + 7 sum_i |n32_i| (|pr_i| + ex_i)
// with sigma = max over faces of sum_i A_i |n_i|.  The row carries slack >= 32 eps sigma
// (rounded up) and thr32 >= thr (1 + 2^-22) (rounded up), and the kernel classifies with
// M = fl32(4u S32 + fl32(thr32 + slack)) (S32: S in FP32, within 8u of S)
//     d32 > M -> d64 >= thr (positive);  d32 < -M -> d64 <= -thr (negative);
// anything else (including NaN) falls back to the exact FP64 distance of that face.
// The cells, statuses and walk paths are therefore the reference's for the position.
// Fallbacks are counted.  The hot loop issues no FP64 instruction.
//
// Positions.  The precision forms hold each coordinate as a float pair (hi, lo) whose exact
// sum is the position.  The plain form walks its FP64 position x through its split
// (hi = fl32(x), lo = fl32(x - hi), within 2^-48 |x| <= u ex of x): that offset adds at most
// u sum_i |n_i| ex_i to the error, well inside the 7 sum_i |n32_i| ex_i of S, and the undecided
// faces are computed from x itself (EXACT), so every class is x's own.
//
// Per-cell FP32 row (128 B, one cache line, 8 x 16 B): c0h (3 x f32), thr32 (f32, negative for
// a degenerate cell), c0l (3 x f32), slack (f32), then per face LEFT..BACK: n32 (3 x f32), e32.
#pragma once
#include "fdf_internal.cuh"
#include "fdf_exact.cuh"

namespace {

using fdfx::add;
using fdfx::mul;
using fdfx::sub;

__device__ __forceinline__ double pair_value(float2 p) { return __dadd_rn((double)p.x, (double)p.y); }

// Exact FP64 signed distance of face f (the plain path's arithmetic), thresholded.
__device__ __forceinline__ double exact_face(const double *__restrict__ row64, int f, double x, double y, double z) {
  const double2 *r = reinterpret_cast<const double2 *>(row64);
  double2 p0 = __ldg(r + 3 * f), p1 = __ldg(r + 3 * f + 1), p2 = __ldg(r + 3 * f + 2);
  double2 tf = __ldg(r + 18);
  double dd = add(add(mul(sub(p0.x, x), p1.y), mul(sub(p0.y, y), p2.x)), mul(sub(p1.x, z), p2.y));
  if (fdfx::abs_lt_bits(dd, fdfx::ubits(tf.x), fdfx::is_nan(tf.x))) dd = 0.0;
  return dd;
}

// The exact distance out of line: the face the FP32 bound cannot decide is rare (about 1e-5
// per particle-step), and kept inline the compiler if-converts it, so every face of every
// evaluation issues its FP64 instructions predicated off (the FP32 walk: 3.91 -> 3.65 ms per
// 64M-particle step out of line).
static __device__ __noinline__ double exact_face_call(const double *__restrict__ row64, int f, double x, double y,
                                                      double z) {
  return exact_face(row64, f, x, y, z);
}
static __device__ __noinline__ double exact_face_pair(const double *__restrict__ row64, int f, float2 px, float2 py,
                                                      float2 pz) {
  return exact_face(row64, f, pair_value(px), pair_value(py), pair_value(pz));
}

// One cell evaluated for the form's position: the face classes the walk needs and the
// distances the weights use.
struct Eval32 {
  unsigned int neg;   // bit f: face f negative
  bool zero;          // some face within its threshold
  bool degenerate;
  float dv[6];
};

// EXACT: the position is the FP64 (xe, ye, ze) and the pairs are its split (hi = fl32(x),
// lo = fl32(x - hi), within 2^-48 |x| of it, which the margin's slack covers); the faces the
// FP32 bound cannot decide are then computed from the FP64 position itself.
template <bool EXACT = false>
__device__ __forceinline__ void eval_cell32(const float *__restrict__ table, const double *__restrict__ planes,
                                            long long cur, float2 px, float2 py, float2 pz, float sx, float sy,
                                            float sz, Eval32 &e, unsigned int &fb, double xe = 0.0,
                                            double ye = 0.0, double ze = 0.0) {
  const float4 *row = reinterpret_cast<const float4 *>(table + cur * FDF_ROW32);
  const float4 h0 = __ldg(row), h1 = __ldg(row + 1);
  e.neg = 0u;
  e.zero = false;
  e.degenerate = (__float_as_uint(h0.w) >> 31) != 0u;
  if (e.degenerate) return;
  float4 fr[6];   // per face: n32 (x, y, z), e32 (w); six 16-B loads
#pragma unroll
  for (int q = 0; q < 6; ++q) fr[q] = __ldg(row + 2 + q);
  const float prx = __fadd_rn(__fsub_rn(px.x, h0.x), __fsub_rn(px.y, h1.x));
  const float pry = __fadd_rn(__fsub_rn(py.x, h0.y), __fsub_rn(py.y, h1.y));
  const float prz = __fadd_rn(__fsub_rn(pz.x, h0.z), __fsub_rn(pz.y, h1.z));
  // |pr_i| + ex_i, ex_i = u (|ph_i| + |c0h_i|): the split term of the bound
  const float ax = __fmaf_rn(__fadd_rn(sx, fabsf(h0.x)), 5.9604644775390625e-8f, fabsf(prx));
  const float ay = __fmaf_rn(__fadd_rn(sy, fabsf(h0.y)), 5.9604644775390625e-8f, fabsf(pry));
  const float az = __fmaf_rn(__fadd_rn(sz, fabsf(h0.z)), 5.9604644775390625e-8f, fabsf(prz));
  const float base = __fadd_rn(h0.w, h1.w);   // thr32 + slack
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    const float nx = fr[f].x, ny = fr[f].y, nz = fr[f].z, ef = fr[f].w;
    const float d32 = __fsub_rn(ef, __fmaf_rn(nz, prz, __fmaf_rn(ny, pry, __fmul_rn(nx, prx))));
    const float S = __fmaf_rn(7.0f, __fmaf_rn(fabsf(nz), az, __fmaf_rn(fabsf(ny), ay, __fmul_rn(fabsf(nx), ax))),
                              __fadd_rn(fabsf(ef), fabsf(ef)));
    const float M = __fmaf_rn(S, 4.0f * 5.9604644775390625e-8f, base);
    if (d32 > M) {
      e.dv[f] = d32;
    } else if (d32 < -M) {
      e.neg |= 1u << f;
      e.dv[f] = d32;
    } else {
      const double d64 = EXACT ? exact_face_call(planes + cur * FDF_ROW, f, xe, ye, ze)
                               : exact_face_pair(planes + cur * FDF_ROW, f, px, py, pz);
      if (fdfx::lt0(d64)) e.neg |= 1u << f;
      e.zero = e.zero || fdfx::eq0(d64);
      e.dv[f] = fdfx::d2f_rn(d64);
      ++fb;
    }
  }
}

// The reference walk from (i, j, k) for at most `limit` evaluations, with Brent cycle
// detection (a revisited cell repeats forever, which the reference ends as LOST after
// MAX_TRAVERSAL evaluations).
struct Walk32 {
  int i, j, k, steps, evaluated;
  bool concluded, lost, cycle;
  unsigned int err;
  Eval32 e;
};

// The cell a walk from (i0, j0, k0) toward (ti, tj, tk) reaches after q steps if every step moves
// each index one closer (the reference's steps move each index by at most one).
__device__ __forceinline__ int path_index(int a0, int t, int q) { return a0 + max(-q, min(q, t - a0)); }

// TRACK: counts in *hits the evaluations after the first whose cell is the one the predicted
// path from the start toward (ti, tj, tk) reaches after as many steps (the rows fetched ahead).
template <bool EXACT = false, bool TRACK = false>
__device__ __forceinline__ void walk_ref32(const float *__restrict__ table, const double *__restrict__ planes,
                                           const GridDims &g, float2 px, float2 py, float2 pz, int limit, Walk32 &w,
                                           unsigned int &fb, double xe = 0.0, double ye = 0.0, double ze = 0.0,
                                           int ti = 0, int tj = 0, int tk = 0, unsigned int *hits = nullptr) {
  const float sx = fabsf(px.x), sy = fabsf(py.x), sz = fabsf(pz.x);
  long long saved = -1;
  int power = 1, lam = 0;
  const int i0 = w.i, j0 = w.j, k0 = w.k;
  w.steps = 0; w.evaluated = 0;
  w.concluded = false; w.lost = false; w.cycle = false;
  while (!w.concluded && w.steps < limit) {
    ++w.steps;
    if (w.i < 0 || w.i >= g.IM || w.j < 0 || w.j >= g.JM || w.k < 0 || w.k >= g.KM) { w.lost = true; break; }
    const long long cur = ((long long)w.k * g.JM + w.j) * g.IM + w.i;
    if (cur == saved) { w.cycle = true; w.lost = true; break; }
    if (++lam == power) { saved = cur; power <<= 1; lam = 0; }
    if (TRACK && w.steps > 1) {
      const int q = w.steps - 1;
      *hits += (w.i == path_index(i0, ti, q) && w.j == path_index(j0, tj, q) && w.k == path_index(k0, tk, q)) ? 1u : 0u;
    }
    eval_cell32<EXACT>(table, planes, cur, px, py, pz, sx, sy, sz, w.e, fb, xe, ye, ze);
    if (w.e.degenerate) { w.err |= ERRBIT_DEGENERATE; w.lost = true; break; }
    ++w.evaluated;
    if (!w.e.neg || w.e.zero) {
      w.concluded = true;
    } else {
      const unsigned int ng = w.e.neg;
      if (ng & (1u << F_FRONT)) w.k += 1; else if (ng & (1u << F_BACK)) w.k -= 1;
      if (ng & (1u << F_LEFT)) w.i -= 1; else if (ng & (1u << F_RIGHT)) w.i += 1;
      if (ng & (1u << F_BOTTOM)) w.j -= 1; else if (ng & (1u << F_TOP)) w.j += 1;
    }
  }
}

}  // namespace
