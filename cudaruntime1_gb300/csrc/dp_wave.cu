// dp_wave.cu -- band-relative anti-diagonal DP for DTW and discrete Frechet:
// a warp per (query, candidate) pair, lane p holding the p-th live cell of
// the current anti-diagonal (R cells per lane for anti-diagonals of up to
// 32 R live cells).  The latency form of the DP: a round of few pairs lasts
// as long as its longest pair, whose n+m-1 anti-diagonals are its steps --
// and, with the query read through L1 and the remaining columns' LB_Keogh
// bound in its abandon test, DTW's survivor round.
//
// Anti-diagonal t = i + j holds the band's cells i in [ilo(t), ihi(t)]
// (|i(m-1) - j(n-1)| <= W inside the matrix), L(t) of them.  From one
// anti-diagonal to the next ilo advances by s = 0 or 1, the same for the
// whole pair.  Position q of step t is cell (ilo(t) + q, t - ilo(t) - q);
// with s = 0 it moves one column right, with s = 1 one row down:
//   s = 0:  up = position q-1, left = position q,    diag = left of q-1
//   s = 1:  up = position q,   left = position q+1,  diag = left of q
// With M_q = min(V_q, the left value V_q was computed from), a cell is
//   s = 0:  combine(cost, min(M_{q-1}, V_q)),   s = 1:  combine(cost, min(M_q, V_{q+1}))
// -- min(M, V) is the minimum of up, left and diagonal, exact in any order,
// so values are the same bits as the other DP kernels'.  One shuffle per
// step moves the neighbour across lanes: M from the lane above when s = 0,
// V from the lane below when s = 1.  Positions at or past L(t) hold +inf.
//
// Edges: above position 0 lies row ilo(t) - 1, outside the band on
// anti-diagonal t; its left neighbour (position 0's diagonal when s = 0) is
// inside when the previous step had s = 1, and is then position 0's value
// two steps back, which lane 0 keeps.  Below the last position lies +inf.
//
// Per step a lane does: one shuffle, R cells, and the costs of the next
// step's R cells from the pair's points (the candidate staged in shared
// memory, padded so that positions past L read inside the buffer and are
// masked; the query staged too in the latency rounds, else read through L1
// with its index clamped).  The geometry (ilo, L) of the anti-diagonals
// comes from exact integer ramps, 32 steps at a time, one per lane, read by
// a shuffle.  Steps run in straight-line blocks of 16; R (1 or 2) is chosen
// per pair inside one launch.  Early abandon: every warping path crosses one
// of any two consecutive anti-diagonals and values never decrease along a
// path, so after every block the minimum over its last two anti-diagonals
// (plus, in the survivor round, the bound of the columns after them) is
// compared with the query's threshold.
//
// Reference kernels replaced: dtw_refine_kernel (CudaRuntime1/dtw.cu:41-96)
// and frechet_refine_kernel_m (CudaRuntime1/frechet.cu:44-117): a CTA per
// pair, a full anti-diagonal of threads and two barriers per step.
#include <type_traits>
#include <vector>

#include "bounds.cuh"
#include "debug_bounds.cuh"
#include "dp_policies.cuh"

namespace tsim {
namespace {
using namespace dp;

constexpr int kWaveThreads = 128;
constexpr int kWavePad = 64;  // points staged past the ends (positions beyond L read them)
constexpr int kWaveMaxLen = 2048;  // longest trajectory of either side

template <class V>
__device__ __forceinline__ V vmin(V a, V b) {
  return b < a ? b : a;
}
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ df vmin(df a, df b) { return df_min3(a, b, b); }

__device__ __forceinline__ float wshfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ df wshfl(df v, int src) {
  return df{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// the most live cells any anti-diagonal of an n x m pair holds
__host__ __device__ inline int wave_lmax(int n, int m, int w) {
  const int mn = n < m ? n : m;
  if (w < 0 || n < 2 || m < 2) return mn;
  const long long W = (long long)w * (mn - 1);
  const long long l = 2 * W / (n + m - 2) + 1;
  return (int)(l < mn ? l : mn);
}

// float2 slots of shared memory per warp: candidate points (pad + ccap +
// pad), the remaining-columns bounds sfx[0 .. ccap] as floats, and with
// qcap > 0 the query points (qcap + pad)
__host__ __device__ inline size_t wave_per_warp(int ccap, int qcap) {
  return (size_t)(ccap + 2 * kWavePad) + (ccap + 2) / 2 + (qcap > 0 ? qcap + kWavePad : 0);
}

// the remaining-columns bound (DTW, FP32, with the query's row-box table)
template <class P>
__host__ __device__ bool wave_suffix(const DpArgs& a) {
  return (std::is_same<P, PolDtwSq>::value || std::is_same<P, PolDtwEu>::value) &&
         a.qtab != nullptr && a.thr != nullptr && a.max_n > 0 && a.max_n <= 16384;
}

// Geometry of anti-diagonals base .. base+31, one per lane: ilo | L << 16,
// from exact integer ramps of the band's edges,
//   ilo(t) = max(0, t-m+1, ceil((t(n-1) - W) / D)),
//   ihi(t) = min(n-1, t, floor((t(n-1) + W) / D)),  D = n+m-2,
// as quotient and remainder (the lower numerator shifted by K D > W to stay
// non-negative), advanced 16 anti-diagonals at a time.  Past the last
// anti-diagonal L is 0 and ilo runs on past n-1 (those steps' cells are
// never used; their point reads stay inside the buffers).
struct WaveGeom {
  int lq, lr, hq, hr;  // this lane's ramps
  int t;               // this lane's anti-diagonal
  int D, K, sq, sr;    // denominator, shift, 16 (n-1) = sq D + sr
  bool band;
  __device__ __forceinline__ void init(int n, int m, int W, int t0) {
    D = n + m - 2;
    band = W >= 0;
    K = band ? W / D + 1 : 0;
    t = t0;
    sq = 16 * (n - 1) / D;
    sr = 16 * (n - 1) - sq * D;
    lq = lr = hq = hr = 0;
    if (band) {
      const int xl = t * (n - 1) - W + (D - 1) + K * D, xh = t * (n - 1) + W;
      lq = xl / D;
      lr = xl - lq * D;
      hq = xh / D;
      hr = xh - hq * D;
    }
  }
  __device__ __forceinline__ int entry(int n, int m) const {
    int lo = max(0, t - (m - 1)), hi = min(n - 1, t);
    if (band) {
      lo = max(lo, lq - K);
      hi = min(hi, hq);
    }
    return lo | (max(0, hi - lo + 1) << 16);
  }
  __device__ __forceinline__ void advance16() {
    t += 16;
    if (band) {
      lq += sq;
      lr += sr;
      if (lr >= D) lr -= D, ++lq;
      hq += sq;
      hr += sr;
      if (hr >= D) hr -= D, ++hq;
    }
  }
};

// shared-memory views of the staged pair: candidate points [-pad, ccap +
// pad), query points [0, qcap + pad) (QS: staged, else read through L1)
#define CS(j) cs[TSIM_SIDX((j) + kWavePad, ccap + 2 * kWavePad) - kWavePad]
#define SFX(j) sfx[TSIM_SIDX(j, ccap + 1)]
#define QPT(i) (QS ? qs[TSIM_SIDX(i, qcap + kWavePad)] : __ldg(A + min(i, n - 1)))

// One pair on the warp, R cells per lane (its widest anti-diagonal fits 32 R).
template <class P, int R, bool QS>
__device__ __forceinline__ void wave_pair(const DpArgs& a, const int pid, const int q, const int n,
                                          const int m, const int w, const int64_t qo,
                                          const int64_t co, float2* cs, float* sfx, float2* qs,
                                          const int ccap, const int qcap) {
  using V = typename P::V;
  using C = typename P::C;
  const int lane = threadIdx.x & 31;
  const bool check = a.thr != nullptr;
  const int src_dn = (lane + 31) & 31, src_up = (lane + 1) & 31;
  const int t_end = n + m - 2;
  const float thr = check ? a.thr[q] : TSIM_INF;
  const int W = w < 0 ? -1 : w * (min(n, m) - 1);
  // the candidate's points are staged; the query's too in the latency
  // rounds (a lone pair's step waits on them), else read through L1, which
  // every pair of the query shares, for the smaller footprint
  const float2* A = a.qpts + qo;

  __syncwarp();
  {
    const float2* B = a.cpts + co;
    for (int j = lane; j < m; j += 32) CS(j) = __ldg(B + j);
    if (QS)
      for (int i = lane; i < n; i += 32) qs[TSIM_SIDX(i, qcap + kWavePad)] = __ldg(A + i);
  }
  // Remaining-columns bound (the survivor round): every path crosses every
  // column after the largest one of two consecutive anti-diagonals, and a
  // cell of column j costs at least the distance from candidate point j to
  // the box of the query rows j's band admits.  sfx[j] = those bounds summed
  // over columns j .. m-1 (rounded down; sfx[m] = 0).  The FP32 path sum that
  // adds those columns' costs can round below their exact sum by at most
  // (n+m+8) 2^-24 relative, so the check compares with the threshold divided
  // by 1 minus that.
  const bool suffix = wave_suffix<P>(a) && n <= a.max_n;
  float thr_chk = thr;
  __syncwarp();
  if (suffix) {
    const QTable T = qtable_view(a.qtab + (size_t)q * qtable_stride(a.max_n), n);
    float carry = 0.0f;  // bound of the columns after the current block
    for (int b0 = ((m - 1) >> 5) << 5; b0 >= 0; b0 -= 32) {  // blocks of 32 columns, last first
      const int j = b0 + lane;
      float v = 0.0f;
      if (j < m) {
        int lo = 0, hi = n - 1;
        if (W >= 0) {
          lo = max(0, floordiv_i((long long)j * (n - 1) - W + (m - 2), m - 1));  // ceil
          hi = min(n - 1, floordiv_i((long long)j * (n - 1) + W, m - 1));
        }
        if (lo <= hi) {
          const float4 bx = qtable_box(T, lo, hi);
          const float2 c = CS(j);
          v = box_pt_d2_rd(bx.x, bx.y, bx.z, bx.w, c.x, c.y);
          if (std::is_same<P, PolDtwEu>::value) v = __fsqrt_rd(v);
        } else {
          v = TSIM_INF;  // a column with no admissible row: no path
        }
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {  // suffix sums inside the block
        const float u = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v = __fadd_rd(v, u);
      }
      v = __fadd_rd(v, carry);
      if (j < m) SFX(j) = v;
      carry = __shfl_sync(0xffffffffu, v, 0);
    }
    if (lane == 0) SFX(m) = 0.0f;
    const float shrink = __fsub_rd(1.0f, __fmul_ru((float)(n + m + 8), 6.03e-8f));
    thr_chk = __fdiv_ru(thr, shrink);
    __syncwarp();
  }

  __syncwarp();
  // anti-diagonals base .. base + 31 of this block and the next, a lane each
  WaveGeom geo;
  geo.init(n, m, W, 1 + lane);
  int win = geo.entry(n, m);
  int base = 1;

  // step 0: cell (0, 0) at position 0; every other position outside
  V v[R], mm[R];
#pragma unroll
  for (int r = 0; r < R; ++r) v[r] = mm[r] = P::border();
  if (lane == 0) {
    const float2 p = QPT(0), c = CS(0);
    v[0] = P::cell(p.x, p.y, c.x, c.y, P::border(), P::border(), P::origin(), a.eps);
    mm[0] = v[0];  // its left (0, -1) is outside
  }
  // costs of the cells of step tt (positions lane R + r), geometry lo; rows
  // past the query's end (masked positions) read its last point
  auto costs = [&](C* out, int tt, int lo) {
    const int i0 = lo + lane * R, j0 = tt - lo - lane * R;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float2 qp = QPT(i0 + r), cp = CS(j0 - r);
      out[r] = P::cost(qp.x, qp.y, cp.x, cp.y);
    }
  };
  C cst[R];
  int e = __shfl_sync(0xffffffffu, win, 0);   // geometry of the step computed next
  int e1 = __shfl_sync(0xffffffffu, win, 1);  // and of the one after
  costs(cst, 1, e & 0xffff);
  V edge = P::border();  // lane 0: position 0's diagonal when the next shift is 0
  int ilo = 0;
  bool alive = true;
  // one anti-diagonal: the shuffle, R cells, and the next step's costs
  // (computed past the last step too: the padding keeps them in bounds);
  // e2 is the geometry of step t + 2
  auto step = [&](const int t, const int e2) {
    const int nlo = e & 0xffff, L = e >> 16;
    const int s = nlo - ilo;  // 0 or 1, uniform
    // across lanes: s = 0 takes M of the lane above's last position, s = 1
    // V of the lane below's first position
    const V xin = wshfl(s ? v[0] : mm[R - 1], s ? src_up : src_dn);
    C cn[R];
    costs(cn, t + 1, e1 & 0xffff);
    const V edge_next = s ? v[0] : P::border();
    V nv[R], nm[R];  // every position reads the last step's values
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const V mdu0 = r > 0 ? mm[r > 0 ? r - 1 : 0] : (lane == 0 ? edge : xin);
      const V lft1 = r + 1 < R ? v[r + 1 < R ? r + 1 : 0] : (lane == 31 ? P::border() : xin);
      const V mdu = s ? mm[r] : mdu0;
      const V lft = s ? lft1 : v[r];
      const V c = P::combine(cst[r], vmin(mdu, lft));
      const bool in = lane * R + r < L;
      nv[r] = in ? c : P::border();
      nm[r] = in ? vmin(c, lft) : P::border();
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r] = nv[r];
      mm[r] = nm[r];
      cst[r] = cn[r];
    }
    edge = edge_next;
    ilo = nlo;
    e = e1;
    e1 = e2;
  };
  auto lane_min = [&]() {
    float x = vf(v[0]);
#pragma unroll
    for (int r = 1; r < R; ++r) x = fminf(x, vf(v[r]));
    return x;
  };
  // blocks of 16 straight-line steps; after each, the abandon test over
  // its last two anti-diagonals (plus the columns after them)
  int t = 1;
  for (; t + 15 <= t_end; t += 16) {
    float m14 = TSIM_INF;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      step(t + u, __shfl_sync(0xffffffffu, win, u + 2));
      if (u == 14) m14 = lane_min();
    }
    geo.advance16();
    const int win_next = geo.entry(n, m);
    if (check) {
      const float two = fminf(lane_min(), m14);
      float lb = __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(two)));
      // the largest column of anti-diagonals t+14, t+15 is t+15 - ilo(t+15)
      if (suffix) lb = __fadd_rd(lb, SFX(min(t + 15 - ilo + 1, m)));
      if (lb > thr_chk) {  // uniform across the warp
        alive = false;
        t += 15;
        break;
      }
    }
    win = win_next;
    base += 16;
  }
  if (alive)
    for (; t <= t_end; ++t) step(t, __shfl_sync(0xffffffffu, win, t + 2 - base));
  if (a.cells) {  // cells of the anti-diagonals computed, inside the band
    const int t_done = alive ? t_end : min(t, t_end);
    long long cells = 0;
    WaveGeom g2;
    g2.init(n, m, W, lane);
    for (int u = lane; u <= t_done; u += 32) {
      cells += g2.entry(n, m) >> 16;
      g2.advance16();
      g2.advance16();
    }
    for (int o = 16; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o);
    if (lane == 0) atomicAdd(a.cells, (unsigned long long)cells);
  }
  // the result: cell (n-1, m-1), position 0 of the last anti-diagonal
  if (lane == 0) store_result(a, pid, alive ? v[0] : P::border());
}

// RMAX = 1: pairs whose widest anti-diagonal fits 32 lanes; RMAX = 2: every
// pair up to 64 cells per anti-diagonal, each with the R (1 or 2) it needs --
// one launch instead of a pass per R (the passes would run one after the
// other, each as long as its longest pair)
template <class P, int RMAX, bool QS>
__global__ void __launch_bounds__(kWaveThreads)
    dp_wave_kernel(DpArgs a, int ccap, int qcap, int* spill, int* nspill) {
  static_assert(P::kMin, "the band-relative kernel serves the minimum measures");
  extern __shared__ __align__(16) float2 wave_smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  float2* cs = wave_smem + (size_t)warp * wave_per_warp(ccap, QS ? qcap : 0) +
               kWavePad;  // cs[-pad .. ccap + pad)
  float* sfx = reinterpret_cast<float*>(cs + ccap + kWavePad);
  float2* qs = cs + ccap + kWavePad + (ccap + 2) / 2;  // QS: qs[0 .. qcap + pad)
  const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nslots = (gridDim.x * blockDim.x) >> 5;
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;

  for (int wk = slot; wk < npairs; wk += nslots) {
    const int pid = a.order ? a.order[wk] : wk;
    const int2 pr = a.pairs[pid];
    if (pr.y < 0) continue;
    const int q = pr.x;
    const int64_t qo = a.qoff[q], co = a.coff[pr.y];
    const int n = (int)(a.qoff[q + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    const int w = band_w(n, m, a.band_pct);
    const int lm = wave_lmax(n, m, w);
    if (n < 2 || m < 2 || n > (QS ? qcap : kWaveMaxLen) || m > ccap || lm > 32 * RMAX) {
      if (lane == 0 && spill) spill[atomicAdd(nspill, 1)] = pid;
      continue;
    }
    if (RMAX == 1 || lm <= 32)  // uniform across the warp
      wave_pair<P, 1, QS>(a, pid, q, n, m, w, qo, co, cs, sfx, qs, ccap, qcap);
    else
      wave_pair<P, RMAX, QS>(a, pid, q, n, m, w, qo, co, cs, sfx, qs, ccap, qcap);
  }
}

#undef CS
#undef SFX
#undef QPT

template <class P, int R, bool QS>
int launch_wave_one(tsim_ctx* ctx, const DpArgs& a, int ccap, int qcap, int* spill, int* nspill) {
  if (a.npairs <= 0) return TSIM_OK;
  auto kern = dp_wave_kernel<P, R, QS>;
  const size_t smem =
      (size_t)(kWaveThreads / 32) * wave_per_warp(ccap, QS ? qcap : 0) * sizeof(float2);
  if (smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWaveThreads, smem));
  if (per_sm < 1) return fail(TSIM_ERR_UNSUPPORTED, "wave kernel does not fit on an SM");
  const long long warps = kWaveThreads / 32;
  const long long blocks = std::min<long long>((a.npairs + warps - 1) / warps,
                                               (long long)per_sm * ctx->num_sms);
  kern<<<(unsigned)std::max(blocks, 1ll), kWaveThreads, smem, ctx->stream>>>(a, ccap, qcap, spill,
                                                                             nspill);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

template <class P>
int wave_chain(tsim_ctx* ctx, const DpArgs& a, int max_n, int max_m, bool latency, int* spill,
               int* nspill) {
  // one launch: R = 1 for the pairs whose widest anti-diagonal fits 32
  // lanes, R = 2 for the others (the longest lengths give the widest band);
  // pairs longer than the staging capacity or wider than 64 cells per
  // anti-diagonal are left in spill.  Latency rounds stage the query too.
  const int ccap = (std::min(max_m, kWaveMaxLen) + 1) & ~1;
  const int qcap = (std::min(max_n, kWaveMaxLen) + 1) & ~1;
  const int lmax = wave_lmax(max_n, max_m, band_w(max_n, max_m, a.band_pct));
  TSIM_CUDA(cudaMemsetAsync(nspill, 0, sizeof(int), ctx->stream));
  if (latency)
    return lmax <= 32 ? launch_wave_one<P, 1, true>(ctx, a, ccap, qcap, spill, nspill)
                      : launch_wave_one<P, 2, true>(ctx, a, ccap, qcap, spill, nspill);
  return lmax <= 32 ? launch_wave_one<P, 1, false>(ctx, a, ccap, qcap, spill, nspill)
                    : launch_wave_one<P, 2, false>(ctx, a, ccap, qcap, spill, nspill);
}

}  // namespace

bool wave_kind(int kind) {
  return kind == DP_DTW_SQ || kind == DP_DTW_EU || kind == DP_FRECHET_SQ || kind == DP_DTW_SQC ||
         kind == DP_DTW_EUC || kind == DP_FRECHET_SQC;
}

int launch_dp_wave(tsim_ctx* ctx, int kind, const DpArgs& a, int max_n, int max_m, bool latency,
                   int* spill, int* nspill) {
  switch (kind) {
    case DP_DTW_SQ: return wave_chain<PolDtwSq>(ctx, a, max_n, max_m, latency, spill, nspill);
    case DP_DTW_EU: return wave_chain<PolDtwEu>(ctx, a, max_n, max_m, latency, spill, nspill);
    case DP_FRECHET_SQ:
      return wave_chain<PolFrechetSq>(ctx, a, max_n, max_m, latency, spill, nspill);
    case DP_DTW_SQC: return wave_chain<PolDtwSqC>(ctx, a, max_n, max_m, latency, spill, nspill);
    case DP_DTW_EUC: return wave_chain<PolDtwEuC>(ctx, a, max_n, max_m, latency, spill, nspill);
    case DP_FRECHET_SQC:
      return wave_chain<PolFrechetSqC>(ctx, a, max_n, max_m, latency, spill, nspill);
  }
  return fail(TSIM_ERR_UNSUPPORTED, "no band-relative kernel for this DP kind");
}

}  // namespace tsim
