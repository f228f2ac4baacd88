// dfloat.cuh -- compensated FP32 arithmetic (an unevaluated sum hi + lo of
// two floats) for the re-score of the top-k survivors.
//
// Error-free transformations: TwoSum (Knuth), Fast2Sum (Dekker, |a| >= |b|)
// and the FMA product error.  A DP value carried as (hi, lo) accumulates its
// rounding errors in lo, so the sum along a DTW path of P cells adds only
// O(P u^2) (u = 2^-24) to the error of its terms instead of P u; the FP32
// pipes issue these far faster than FP64 on this GPU.
#pragma once
#include "tsim_internal.cuh"

namespace tsim {

struct df {
  float hi, lo;
};

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum_f(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df df_inf() { return df{TSIM_INF, 0.0f}; }

// lexicographic order of normalised pairs = order of the values they represent
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ df df_min(df a, df b) { return df_lt(b, a) ? b : a; }
__device__ __forceinline__ df df_max(df a, df b) { return df_lt(a, b) ? b : a; }

// (qx - cx)^2 + (qy - cy)^2 as a normalised pair, relative error <= ~10 u^2
__device__ __forceinline__ df df_sqdist(float qx, float qy, float cx, float cy) {
  float dxh, dxl, dyh, dyl;
  two_sum_f(qx, -cx, dxh, dxl);
  two_sum_f(qy, -cy, dyh, dyl);
  const float px = __fmul_rn(dxh, dxh), pex = __fmaf_rn(dxh, dxh, -px);
  const float py = __fmul_rn(dyh, dyh), pey = __fmaf_rn(dyh, dyh, -py);
  const float cross = __fmul_rn(2.0f, __fmaf_rn(dxh, dxl, __fmul_rn(dyh, dyl)));
  float s, e;
  two_sum_f(px, py, s, e);
  const float lo = __fadd_rn(__fadd_rn(e, __fadd_rn(pex, pey)), cross);
  return fast_two_sum_f(s, lo);
}

// a + b for normalised, finite, non-negative pairs
__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum_f(a.hi, b.hi, s, e);
  return fast_two_sum_f(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

// c + b for a float c >= 0 and a normalised, finite, non-negative pair b
__device__ __forceinline__ df df_add1(float c, df b) {
  float s, e;
  two_sum_f(c, b.hi, s, e);
  return fast_two_sum_f(s, __fadd_rn(e, b.lo));
}

// sqrt of a normalised non-negative pair: one Newton correction of sqrtf(hi)
__device__ __forceinline__ df df_sqrt(df a) {
  if (a.hi <= 0.0f) return df{0.0f, 0.0f};
  const float s = __fsqrt_rn(a.hi);
  const float r = __fadd_rn(__fmaf_rn(-s, s, a.hi), a.lo);  // exact residual + lo
  return fast_two_sum_f(s, __fdiv_rn(r, __fmul_rn(2.0f, s)));
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

}  // namespace tsim
