// dp_policies.cuh -- cell policies and helpers shared by the wavefront DP
// kernels (dp_kernels.cu: round-striped; dp_diag.cu: anti-diagonal).
#pragma once
#include "dfloat.cuh"
#include "tsim_internal.cuh"

namespace tsim {
namespace dp {

// min of three floats in one instruction (the three-operand PTX min.f32 of
// sm_100+; exact, like two fminf, for the non-NaN values of a DP)
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// q - c per coordinate in one packed instruction (sub.rn.f32x2, sm_100 and
// later): two round-to-nearest subtractions, the bits of two scalar ones
__device__ __forceinline__ float2 sub2(float2 q, float2 c) {
  union {
    float2 f;
    unsigned long long u;
  } a, b, r;
  a.f = q;
  b.f = c;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(a.u), "l"(b.u));
  return r.f;
}

// Minimum of three normalised pairs.  A normalised pair's hi is its value
// rounded to nearest, so pairs with different hi order as their hi parts;
// among the operands whose hi is the smallest, the smallest lo decides.
// Equal to two lexicographic minima, in fewer instructions.
__device__ __forceinline__ df df_min3(df a, df b, df c) {
  const float h = min3f(a.hi, b.hi, c.hi);
  const float la = a.hi == h ? a.lo : TSIM_INF;
  const float lb = b.hi == h ? b.lo : TSIM_INF;
  const float lc = c.hi == h ? c.lo : TSIM_INF;
  return df{h, min3f(la, lb, lc)};
}

// ---- cell policies ---------------------------------------------------------
// V: value type; border(): value outside the matrix / band; origin(): D(-1,-1);
// masked(left): value of a cell outside its row's band.  The minimum
// policies also split a cell into cost() and combine(cost, m), m the minimum
// of up, left and diagonal: cell() == combine(cost(), min3(...)), operation
// for operation (the band-relative kernel computes costs a step ahead).

struct PolDtwRef {  // CudaRuntime1/dtw.cpp:88-93 arithmetic, bit for bit
  using V = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return TSIM_INF; }
  __device__ static V origin() { return 0.0f; }
  __device__ static V masked(V) { return TSIM_INF; }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    float dx = qx - cx, dy = qy - cy;
    float c = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    return __fadd_rn(c, fminf(fminf(up, lf), dg));
  }
};

struct PolFrechetRef {  // CudaRuntime1/frechet.cpp:72-76, 103-108
  using V = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return TSIM_INF; }
  __device__ static V origin() { return 0.0f; }
  __device__ static V masked(V) { return TSIM_INF; }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    float dx = qx - cx, dy = qy - cy;
    float d = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    return fmaxf(d, fminf(fminf(up, lf), dg));
  }
};

struct PolDtwSq {  // squared cost; FMA allowed, error bounded by the caller
  using V = float;
  using C = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return TSIM_INF; }
  __device__ static V origin() { return 0.0f; }
  __device__ static V masked(V) { return TSIM_INF; }
  __device__ static C cost(float qx, float qy, float cx, float cy) {
    float dx = qx - cx, dy = qy - cy;
    return fmaf(dy, dy, dx * dx);
  }
  __device__ static V combine(C c, V m) { return c + m; }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    float dx = qx - cx, dy = qy - cy;
    float c = fmaf(dy, dy, dx * dx);
    return c + min3f(up, lf, dg);
  }
  // cell() with the points as pairs: the same operations, the two
  // differences in one packed subtraction
  __device__ static V cellp(float2 q, float2 p, V up, V lf, V dg, float) {
    const float2 d = sub2(q, p);
    return fmaf(d.y, d.y, d.x * d.x) + min3f(up, lf, dg);
  }
};

struct PolDtwEu {
  using V = float;
  using C = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return TSIM_INF; }
  __device__ static V origin() { return 0.0f; }
  __device__ static V masked(V) { return TSIM_INF; }
  __device__ static C cost(float qx, float qy, float cx, float cy) {
    float dx = qx - cx, dy = qy - cy;
    return sqrtf(fmaf(dy, dy, dx * dx));
  }
  __device__ static V combine(C c, V m) { return c + m; }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    float dx = qx - cx, dy = qy - cy;
    float c = sqrtf(fmaf(dy, dy, dx * dx));
    return c + min3f(up, lf, dg);
  }
  __device__ static V cellp(float2 q, float2 p, V up, V lf, V dg, float) {
    const float2 d = sub2(q, p);
    return sqrtf(fmaf(d.y, d.y, d.x * d.x)) + min3f(up, lf, dg);
  }
};

struct PolFrechetSq {  // squared domain; sqrt is applied once at the end
  using V = float;
  using C = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return TSIM_INF; }
  __device__ static V origin() { return 0.0f; }
  __device__ static V masked(V) { return TSIM_INF; }
  __device__ static C cost(float qx, float qy, float cx, float cy) {
    float dx = qx - cx, dy = qy - cy;
    return fmaf(dy, dy, dx * dx);
  }
  __device__ static V combine(C c, V m) { return fmaxf(c, m); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    float dx = qx - cx, dy = qy - cy;
    float d2 = fmaf(dy, dy, dx * dx);
    return fmaxf(d2, min3f(up, lf, dg));
  }
  __device__ static V cellp(float2 q, float2 p, V up, V lf, V dg, float) {
    const float2 d = sub2(q, p);
    return fmaxf(fmaf(d.y, d.y, d.x * d.x), min3f(up, lf, dg));
  }
};

// FP64 re-score policies: the arithmetic of the FP64 oracle
// (oracle/oracle.c dtw64_core / orc_frechet64), so values are bit-identical
// to it: dx = (double)a - (double)b, cost = dx*dx + dy*dy without FMA.
__device__ __forceinline__ double d2_64(float qx, float qy, float cx, float cy) {
  double dx = (double)qx - (double)cx, dy = (double)qy - (double)cy;
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}
__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }

struct PolDtwSq64 {
  using V = double;
  static constexpr bool kMin = true;
  __device__ static V border() { return __longlong_as_double(0x7ff0000000000000ll); }
  __device__ static V origin() { return 0.0; }
  __device__ static V masked(V) { return border(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    return __dadd_rn(d2_64(qx, qy, cx, cy), dmin(dmin(up, lf), dg));
  }
};

struct PolDtwEu64 {
  using V = double;
  static constexpr bool kMin = true;
  __device__ static V border() { return __longlong_as_double(0x7ff0000000000000ll); }
  __device__ static V origin() { return 0.0; }
  __device__ static V masked(V) { return border(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    return __dadd_rn(__dsqrt_rn(d2_64(qx, qy, cx, cy)), dmin(dmin(up, lf), dg));
  }
};

struct PolFrechetSq64 {
  using V = double;
  static constexpr bool kMin = true;
  __device__ static V border() { return __longlong_as_double(0x7ff0000000000000ll); }
  __device__ static V origin() { return 0.0; }
  __device__ static V masked(V) { return border(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    double d = d2_64(qx, qy, cx, cy), mn = dmin(dmin(up, lf), dg);
    return d > mn ? d : mn;
  }
};

// Exact FP64 discrete Frechet (squared) without an FP64 DP.  A Frechet
// value is a min over paths of a max over cells, so it equals one cell's
// cost.  With FP32 costs d32 (the FP32 DP's arithmetic) and FP64 costs d64
// (the FP64 oracle's), |d32 - d64| <= 8u d64 for normal numbers (u = 2^-24),
// so the FP64 optimum v64 lies within 16u of the pair's FP32 optimum v32
// (passed as the pair's aux value).  A cell whose d32 is at most v32 (1 - 32u)
// has d64 below v64: taking its cost as 0 cannot change any path's maximum
// that could be the optimum; one whose d32 is at least v32 (1 + 32u) has d64
// above v64 and cannot lie on an optimal path, so it is blocked.  Only the
// cells between get their FP64 cost, computed as the oracle does.  Values are
// the bit patterns of non-negative doubles, whose unsigned order is the
// doubles' order: min and max run on the integer ALU, not the FP64 units.
// Below v32 = 1e-20 (FP32 underflow voids the relative bound) every cell
// gets its FP64 cost.
struct PolFrechetWin {
  using V = unsigned long long;
  static constexpr bool kMin = true;
  __device__ static V border() { return 0x7ff0000000000000ull; }  // +inf
  __device__ static V origin() { return 0ull; }                   // +0
  __device__ static V masked(V) { return border(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float v32) {
    const V mn = umin(umin(up, lf), dg);
    const float dx = qx - cx, dy = qy - cy;
    const float d = fmaf(dy, dy, dx * dx);
    const bool exact = !(v32 >= 1e-20f);
    V c;
    if (!exact && d <= __fmul_rd(v32, 1.0f - 32.0f / 16777216.0f)) {
      c = 0ull;  // below any candidate optimum
    } else if (!exact && d >= __fmul_ru(v32, 1.0f + 32.0f / 16777216.0f)) {
      c = border();  // above it
    } else {
      c = (V)__double_as_longlong(d2_64(qx, qy, cx, cy));
    }
    return c > mn ? c : mn;
  }
  __device__ static V umin(V a, V b) { return b < a ? b : a; }
};

// Compensated FP32 re-score policies: values are (hi, lo) pairs (dfloat.cuh).
// DTW: each cell cost in FP32 (<= 4u relative error, one FMA), the path sum
// compensated; the value is then within 4u + O(P u^2) of exact -- a single
// cost's rounding, not P of them.
struct PolDtwSqC {
  using V = df;
  using C = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return df_inf(); }
  __device__ static V origin() { return df{0.0f, 0.0f}; }
  __device__ static V masked(V) { return df_inf(); }
  __device__ static C cost(float qx, float qy, float cx, float cy) {
    const float dx = qx - cx, dy = qy - cy;
    return fmaf(dy, dy, dx * dx);
  }
  __device__ static V combine(C c, V m) { return m.hi < TSIM_INF ? df_add1(c, m) : df_inf(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    const df m = df_min3(up, lf, dg);
    if (!(m.hi < TSIM_INF)) return df_inf();
    const float dx = qx - cx, dy = qy - cy;
    return df_add1(fmaf(dy, dy, dx * dx), m);
  }
};

struct PolDtwEuC {
  using V = df;
  using C = float;
  static constexpr bool kMin = true;
  __device__ static V border() { return df_inf(); }
  __device__ static V origin() { return df{0.0f, 0.0f}; }
  __device__ static V masked(V) { return df_inf(); }
  __device__ static C cost(float qx, float qy, float cx, float cy) {
    const float dx = qx - cx, dy = qy - cy;
    return sqrtf(fmaf(dy, dy, dx * dx));
  }
  __device__ static V combine(C c, V m) { return m.hi < TSIM_INF ? df_add1(c, m) : df_inf(); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    const df m = df_min3(up, lf, dg);
    if (!(m.hi < TSIM_INF)) return df_inf();
    const float dx = qx - cx, dy = qy - cy;
    return df_add1(sqrtf(fmaf(dy, dy, dx * dx)), m);
  }
};

struct PolFrechetSqC {
  using V = df;
  using C = df;
  static constexpr bool kMin = true;
  __device__ static V border() { return df_inf(); }
  __device__ static V origin() { return df{0.0f, 0.0f}; }
  __device__ static V masked(V) { return df_inf(); }
  __device__ static C cost(float qx, float qy, float cx, float cy) { return df_sqdist(qx, qy, cx, cy); }
  __device__ static V combine(C c, V m) { return df_max(c, m); }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float) {
    return df_max(df_sqdist(qx, qy, cx, cy), df_min3(up, lf, dg));
  }
};

// LCSS: match iff |q.x-c.x| < eps and |q.y-c.y| < eps in FP32 (lcss.cpp:93-96).
// Outside the index window a cell keeps its row's last in-window value (the
// true LCSS value there); left of the window it stays 0.  The non-match case
// takes max(up, left, diag), which equals max(up, left) inside the matrix and
// is exact at the window edges where a neighbour lies outside.
struct PolLcss {
  using V = int;
  static constexpr bool kMin = false;
  __device__ static V border() { return 0; }
  __device__ static V origin() { return 0; }
  __device__ static V masked(V lf) { return lf; }
  __device__ static V cell(float qx, float qy, float cx, float cy, V up, V lf, V dg, float eps) {
    bool match = (fabsf(qx - cx) < eps) && (fabsf(qy - cy) < eps);
    return match ? dg + 1 : max(max(up, lf), dg);
  }
  __device__ static V cellp(float2 q, float2 p, V up, V lf, V dg, float eps) {
    const float2 d = sub2(q, p);
    const bool match = (fabsf(d.x) < eps) && (fabsf(d.y) < eps);
    return match ? dg + 1 : max(max(up, lf), dg);
  }
};

// Row whose last in-band value is the pair's result: (n-1, m-1) for DTW and
// Frechet.  For windowed LCSS with n-1 > m-1+delta the last row is empty and
// L(n-1, m-1) = L(m-1+delta, m-1), which the row m-1+delta holds.
template <class P>
__device__ __forceinline__ int result_row(int n, int m, int delta) {
  return n - 1;
}
template <>
__device__ __forceinline__ int result_row<PolLcss>(int n, int m, int delta) {
  return delta >= 0 ? min(n - 1, m - 1 + delta) : n - 1;
}

template <class P>
struct RowBand {
  __device__ __forceinline__ static void get(int i, int n, int m, int w, int, int& lo, int& hi) {
    band_row(i, n, m, w, lo, hi);
  }
};
template <>
struct RowBand<PolLcss> {
  __device__ __forceinline__ static void get(int i, int, int m, int, int delta, int& lo, int& hi) {
    window_row(i, m, delta, lo, hi);
  }
};

__device__ __forceinline__ void store_result(const DpArgs& a, int pid, float v) { a.out[pid] = v; }
__device__ __forceinline__ void store_result(const DpArgs& a, int pid, int v) { a.out[pid] = (float)v; }
__device__ __forceinline__ void store_result(const DpArgs& a, int pid, double v) { a.out64[pid] = v; }
__device__ __forceinline__ void store_result(const DpArgs& a, int pid, unsigned long long v) {
  a.out64[pid] = __longlong_as_double((long long)v);  // the bits of a double
}
__device__ __forceinline__ void store_result(const DpArgs& a, int pid, df v) {
  a.out64[pid] = v.hi < TSIM_INF ? df_to_double(v) : __longlong_as_double(0x7ff0000000000000ll);
}
__device__ __forceinline__ float vf(float v) { return v; }
__device__ __forceinline__ float vf(int v) { return (float)v; }
__device__ __forceinline__ float vf(double v) { return (float)v; }
__device__ __forceinline__ float vf(df v) { return v.hi; }
__device__ __forceinline__ float vf(unsigned long long v) {
  return (float)__longlong_as_double((long long)v);
}

template <class V>
__device__ __forceinline__ V shfl_up_seg(V v, int G) {
  return __shfl_up_sync(0xffffffffu, v, 1, G);
}
template <class V>
__device__ __forceinline__ V shfl_lane(V v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}
__device__ __forceinline__ df shfl_lane(df v, int src) {
  return df{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}
__device__ __forceinline__ df shfl_up_seg(df v, int G) {
  return df{__shfl_up_sync(0xffffffffu, v.hi, 1, G), __shfl_up_sync(0xffffffffu, v.lo, 1, G)};
}

__device__ __forceinline__ float seg_max(float v, int G) {
  for (int o = G >> 1; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o, G));
  return v;
}
__device__ __forceinline__ int seg_max_i(int v, int G) {
  for (int o = G >> 1; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o, G));
  return v;
}


}  // namespace dp
}  // namespace tsim
