// dp_diag.cu -- anti-diagonal wavefront DP for banded / windowed pairs.
//
// One warp per (query, candidate) pair.  Cell (i, j) is computed at step
// t = i + j.  Rows are dealt to lanes in groups of R consecutive rows, round
// robin: lane l owns rows R*(l + 32k) .. R*(l + 32k) + R - 1 for k = 0, 1, ...
// At step t a lane computes column t - i of each row i of its current group,
// so all R cells of a step depend only on the previous step: the row above a
// group (the last row of the previous lane's group) arrives by one register
// shuffle, and there is no shared-memory row buffer and no per-round skew --
// the critical path of a pair is its n + m - 1 anti-diagonals.
//
// A lane moves to its next group when that group's first cell comes up.
// This is valid when a group has finished -- and the next lane has consumed
// its last row -- before the lane's next group starts.  With the band
// |i(m-1) - j(n-1)| <= W (W = w (min(n,m)-1)) that holds whenever
// 2W < 31 R (n + m - 2); for a full row (no band) when m <= 31 R + 1; for
// an LCSS window |i - j| <= delta when delta <= 31 R.  Pairs that fail the
// condition (or whose query exceeds the row table) are listed for the
// round-striped kernel instead (dp_kernels.cu).
//
// Early abandon: every warping path crosses one of any two consecutive
// anti-diagonals and DP values never decrease along a path, so the minimum
// over the last two anti-diagonals bounds the final value from below.
#include "dp_policies.cuh"

namespace tsim {
namespace {
using namespace dp;

constexpr int kDiagThreads = 128;
constexpr int kNone = 1 << 30;

}  // namespace

__host__ __device__ bool diag_ok(bool lcss, int n, int m, int wd, int R) {
  if (n < 2 || m < 2) return false;
  if (wd < 0) return m <= 31 * R + 1;
  if (lcss) return wd <= 31 * R;
  const long long W = (long long)wd * ((n < m ? n : m) - 1);
  return 2 * W < 31ll * R * (n + m - 2);
}

namespace {

template <class P, int R>
__global__ void __launch_bounds__(kDiagThreads) dp_diag_kernel(DpArgs a, int row_cap, int col_cap,
                                                                int* spill, int* nspill) {
  using V = typename P::V;
  extern __shared__ __align__(16) float4 diag_rows[];
  constexpr bool kLcss = !P::kMin;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  // per warp: the row table, then the candidate's points
  float4* rt = diag_rows + (size_t)wib * (row_cap + col_cap / 2);
  float2* cs = reinterpret_cast<float2*>(rt + row_cap);
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;

  for (int wk = gw; wk < npairs; wk += nw) {
    const int pid = a.order ? a.order[wk] : wk;
    const int2 pr = a.pairs[pid];
    if (pr.y < 0) continue;
    const int q = pr.x;
    const int64_t qo = a.qoff[q], co = a.coff[pr.y];
    const int n = (int)(a.qoff[q + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    const float2* A = a.qpts + qo;
    const float2* B = a.cpts + co;
    const int w = band_w(n, m, a.band_pct);
    const int wd = kLcss ? a.delta : w;
    const int nr = (n + 32 * R - 1) / (32 * R) * (32 * R);  // rows incl. padding
    if (!diag_ok(kLcss, n, m, wd, R) || nr > row_cap || m > col_cap) {
      if (lane == 0 && spill) spill[atomicAdd(nspill, 1)] = pid;
      continue;
    }
    const float thr = a.thr ? a.thr[q] : TSIM_INF;
    const int rrow = result_row<P>(n, m, a.delta);
    if (lane == 0) store_result(a, pid, P::border());

    // row table: query point and band of every row (empty rows: kNone)
    long long cells_all = 0;
    for (int i = lane; i < nr; i += 32) {
      float4 e = make_float4(0.f, 0.f, __int_as_float(kNone), __int_as_float(kNone));
      if (i < n) {
        int lo, hi;
        RowBand<P>::get(i, n, m, w, a.delta, lo, hi);
        const float2 p = A[i];
        if (hi >= lo) {
          e = make_float4(p.x, p.y, __int_as_float(lo), __int_as_float(hi));
          cells_all += hi - lo + 1;
        } else {
          e = make_float4(p.x, p.y, __int_as_float(kNone), __int_as_float(kNone));
        }
      }
      rt[i] = e;
    }
    for (int j = lane; j < m; j += 32) cs[j] = B[j];  // the candidate, read once
    __syncwarp();

    int i0 = R * lane;  // first row of the lane's current group
    float qx[R], qy[R];
    int jlo[R], jhi[R];
    V left[R], left2[R];  // each row's values one and two columns back
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float4 e = rt[i0 + r];
      qx[r] = e.x;
      qy[r] = e.y;
      jlo[r] = __float_as_int(e.z);
      jhi[r] = __float_as_int(e.w);
      left[r] = left2[r] = P::border();
    }
    // step at which the next group's first row starts (never, if none)
    auto next_start = [&](int base) -> int {
      const int i1 = base + 32 * R;
      if (i1 >= n) return 0x7fffffff;
      const int lo = __float_as_int(rt[i1].z);
      return lo == kNone ? 0x7fffffff : i1 + lo;
    };
    int ns = next_start(i0);
    V out = P::border();
    V prev_raw = P::border();  // the shuffled value of the previous step
    float2 cw[R];
#pragma unroll
    for (int r = 0; r < R; ++r) cw[r] = cs[0];
    V result = P::border();
    bool holds = false;
    bool alive = true;
    float mprev = TSIM_INF;
    const int t_end = n + m - 2;
    int t_ab = t_end;

    for (int t = 0; t <= t_end; ++t) {
      if (t == ns) {  // this lane's next group starts now
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (i0 + r == rrow) {
            result = left[r];
            holds = true;
          }
        i0 += 32 * R;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const float4 e = rt[i0 + r];
          qx[r] = e.x;
          qy[r] = e.y;
          jlo[r] = __float_as_int(e.z);
          jhi[r] = __float_as_int(e.w);
          left[r] = left2[r] = P::border();
        }
        ns = next_start(i0);
      }
      // the last row of the previous lane's group, one column back: the row
      // above this lane's first row (lane 0's first group reads the virtual
      // row -1 instead, whose only finite cell is D(-1,-1) = origin)
      const V raw = shfl_lane(out, (lane + 31) & 31);
      const bool first = lane == 0 && i0 == 0;
      const V up_in = first ? P::border() : raw;
      const V dg_in = first ? (t == 0 ? P::origin() : P::border()) : prev_raw;
      prev_raw = raw;
#pragma unroll
      for (int r = R - 1; r > 0; --r) cw[r] = cw[r - 1];
      const int j0 = t - i0;
      cw[0] = cs[min(max(j0, 0), m - 1)];
      float mstep = TSIM_INF;
      // row r computes column j0 - r: its up neighbour is row r-1 one step
      // ago and its diagonal neighbour row r-1 two steps ago, so rows are
      // visited last to first before row r-1 is overwritten
#pragma unroll
      for (int r = R - 1; r >= 0; --r) {
        const int j = j0 - r;
        const V lf = left[r];
        const V up = r > 0 ? left[r > 0 ? r - 1 : 0] : up_in;
        const V dg = r > 0 ? left2[r > 0 ? r - 1 : 0] : dg_in;
        V v = P::cell(qx[r], qy[r], cw[r].x, cw[r].y, up, lf, dg, a.eps);
        const bool in = (unsigned)(j - jlo[r]) <= (unsigned)(jhi[r] - jlo[r]);
        v = in ? v : P::masked(lf);
        if (P::kMin) mstep = fminf(mstep, in ? vf(v) : TSIM_INF);
        left2[r] = lf;
        left[r] = v;
      }
      out = left[R - 1];
      if (P::kMin && a.thr) {
        const float two = fminf(mstep, mprev);
        mprev = mstep;
        if ((t & 15) == 15) {
          const unsigned lb = __reduce_min_sync(0xffffffffu, __float_as_uint(two));
          if (__uint_as_float(lb) > thr) {  // uniform across the warp
            alive = false;
            t_ab = t;
            break;
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (i0 + r == rrow) {
        result = left[r];
        holds = true;
      }
    if (a.cells) {
      long long cells = cells_all;
      if (!alive) {  // cells of the anti-diagonals computed before abandoning
        cells = 0;
        for (int i = lane; i < n; i += 32) {
          const float4 e = rt[i];
          const int lo = __float_as_int(e.z), hi = __float_as_int(e.w);
          if (lo == kNone) continue;
          const int h = min(hi, t_ab - i);
          if (h >= lo) cells += h - lo + 1;
        }
      }
      for (int o = 16; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o);
      if (lane == 0) atomicAdd(a.cells, (unsigned long long)cells);
    }
    __syncwarp();
    if (holds) store_result(a, pid, alive ? result : P::border());
    if (!alive && lane == 0) store_result(a, pid, P::border());
    __syncwarp();
  }
}

template <class P, int R>
int launch_diag_one(tsim_ctx* ctx, const DpArgs& a, int max_n, int max_m, int* spill,
                    int* nspill) {
  if (a.npairs <= 0) return TSIM_OK;
  const int row_cap = (max_n + 32 * R - 1) / (32 * R) * (32 * R);
  const int col_cap = (max_m + 1) & ~1;  // even: whole float4 slots
  const int warps = kDiagThreads / 32;
  const size_t smem = (size_t)warps * (row_cap + col_cap / 2) * sizeof(float4);
  if (smem > 200 * 1024) return fail(TSIM_ERR_UNSUPPORTED, "pair too long for the row tables");
  auto kern = dp_diag_kernel<P, R>;
  if (smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kDiagThreads, smem));
  long long blocks = std::min<long long>((a.npairs + warps - 1) / warps,
                                         (long long)std::max(per_sm, 1) * ctx->num_sms);
  kern<<<(unsigned)std::max(blocks, 1ll), kDiagThreads, smem, ctx->stream>>>(a, row_cap, col_cap,
                                                                            spill, nspill);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

template <class P>
int launch_diag_r(tsim_ctx* ctx, int R, const DpArgs& a, int max_n, int max_m, int* spill,
                  int* nspill) {
  switch (R) {
    case 1: return launch_diag_one<P, 1>(ctx, a, max_n, max_m, spill, nspill);
    case 2: return launch_diag_one<P, 2>(ctx, a, max_n, max_m, spill, nspill);
    default: return launch_diag_one<P, 4>(ctx, a, max_n, max_m, spill, nspill);
  }
}

}  // namespace

int launch_dp_diag(tsim_ctx* ctx, int kind, int R, const DpArgs& a, int max_n, int max_m,
                   int* spill, int* nspill) {
  switch (kind) {
    case DP_DTW_SQ: return launch_diag_r<PolDtwSq>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_DTW_EU: return launch_diag_r<PolDtwEu>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_LCSS: return launch_diag_r<PolLcss>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_FRECHET_SQ: return launch_diag_r<PolFrechetSq>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_DTW_SQC: return launch_diag_r<PolDtwSqC>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_DTW_EUC: return launch_diag_r<PolDtwEuC>(ctx, R, a, max_n, max_m, spill, nspill);
    case DP_FRECHET_SQC: return launch_diag_r<PolFrechetSqC>(ctx, R, a, max_n, max_m, spill, nspill);
  }
  return fail(TSIM_ERR_UNSUPPORTED, "no anti-diagonal kernel for this DP kind");
}

}  // namespace tsim
