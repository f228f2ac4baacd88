// bounds.cuh -- lower bounds (upper bounds for LCSS) used to prune pairs
// before the exact computation.  Every bound is computed with directed
// rounding toward the safe side, so in FP32 it never exceeds the exact
// (real-number) value of the measure and a true neighbour is never pruned.
#pragma once
#include "tsim_internal.cuh"

namespace tsim {

// |a - b| rounded down
__device__ __forceinline__ float absdiff_rd(float a, float b) {
  return a >= b ? __fsub_rd(a, b) : __fsub_rd(b, a);
}

// squared point distance, rounded down
__device__ __forceinline__ float pd2_rd(float ax, float ay, float bx, float by) {
  float dx = absdiff_rd(ax, bx), dy = absdiff_rd(ay, by);
  return __fadd_rd(__fmul_rd(dx, dx), __fmul_rd(dy, dy));
}

// squared distance from point (x, y) to box (x0, y0, x1, y1), rounded down
__device__ __forceinline__ float box_pt_d2_rd(float x0, float y0, float x1, float y1, float x,
                                              float y) {
  float dx = x < x0 ? __fsub_rd(x0, x) : (x > x1 ? __fsub_rd(x, x1) : 0.0f);
  float dy = y < y0 ? __fsub_rd(y0, y) : (y > y1 ? __fsub_rd(y, y1) : 0.0f);
  return __fadd_rd(__fmul_rd(dx, dx), __fmul_rd(dy, dy));
}

// squared distance between two boxes (x0, y0, x1, y1), rounded down
__device__ __forceinline__ float box_box_d2_rd(float4 a, float4 b) {
  float dx = a.x > b.z ? __fsub_rd(a.x, b.z) : (b.x > a.z ? __fsub_rd(b.x, a.z) : 0.0f);
  float dy = a.y > b.w ? __fsub_rd(a.y, b.w) : (b.y > a.w ? __fsub_rd(b.y, a.w) : 0.0f);
  return __fadd_rd(__fmul_rd(dx, dx), __fmul_rd(dy, dy));
}

// q = floor(num / den), r = num - q den (0 <= r < den) for den > 0 and a
// quotient that fits an int.  32-bit arithmetic when the numerator fits (a
// 64-bit division is a long software sequence), 64-bit otherwise.
__device__ __forceinline__ void divmod_floor(long long num, int den, int& q, int& r) {
  if (num >= -2147483647ll && num <= 2147483647ll) {
    const int n32 = (int)num;
    int qq = n32 / den, rr = n32 - qq * den;
    if (rr < 0) {
      rr += den;
      qq -= 1;
    }
    q = qq;
    r = rr;
  } else {
    long long qq = num / den, rr = num % den;
    if (rr < 0) {
      rr += den;
      qq -= 1;
    }
    q = (int)qq;
    r = (int)rr;
  }
}
__device__ __forceinline__ int floordiv_i(long long num, int den) {
  int q, r;
  divmod_floor(num, den, q, r);
  return q;
}

// Floor division with a non-negative remainder, for incremental stepping.
struct FloorDiv {
  int q, r, d;
  __device__ __forceinline__ void init(long long num, int den) {
    d = den;
    divmod_floor(num, den, q, r);
  }
  // num += dq * d + dr with 0 <= dr < d
  __device__ __forceinline__ void step(int dq, int dr) {
    q += dq;
    r += dr;
    if (r >= d) {
      r -= d;
      q += 1;
    }
  }
};

// Sparse table of a query for O(1) range boxes: level l holds, for block b,
// the box of blocks [b, b + 2^l).  Block = f consecutive rows (f = 1 for
// queries up to kMaxTable rows, a power of two beyond, which widens boxes and
// keeps the bound valid).
constexpr int kMaxTable = 512;  // sparse-table columns (query rows, downsampled beyond)
struct QTable {
  const float4* t;  // [levels][nb] as (x0, y0, x1, y1)
  int nb, f_log, levels;
};

// box of query rows [lo, hi] (non-empty)
__device__ __forceinline__ float4 qtable_box(const QTable& T, int lo, int hi) {
  const int b0 = lo >> T.f_log, b1 = hi >> T.f_log;
  const int l = 31 - __clz(b1 - b0 + 1);
  const float4 u = T.t[(size_t)l * T.nb + b0], v = T.t[(size_t)l * T.nb + b1 - (1 << l) + 1];
  return make_float4(fminf(u.x, v.x), fminf(u.y, v.y), fmaxf(u.z, v.z), fmaxf(u.w, v.w));
}

// float4 entries of a table buffer for queries of up to max_n rows: the
// table size is not monotone in n (a 512-row query keeps 512 blocks, a
// 600-row one 300 blocks of 2 rows), so the buffer is sized for
// min(max_n, kMaxTable) blocks, whose level count no shorter query exceeds
__host__ __device__ inline int qtable_stride(int max_n) {
  const int nb = max_n < 1 ? 1 : (max_n < kMaxTable ? max_n : kMaxTable);
  int levels = 1;
  while ((1 << levels) <= nb) ++levels;
  return levels * nb;
}

// view of a table built for a query of n rows
__device__ __forceinline__ QTable qtable_view(const float4* t, int n) {
  QTable T;
  int f_log = 0;
  while ((n + (1 << f_log) - 1) >> f_log > kMaxTable) ++f_log;
  T.t = t;
  T.f_log = f_log;
  T.nb = (n + (1 << f_log) - 1) >> f_log;
  int levels = 1;
  while ((1 << levels) <= T.nb) ++levels;
  T.levels = levels;
  return T;
}

}  // namespace tsim
