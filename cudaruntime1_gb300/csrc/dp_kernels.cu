// dp_kernels.cu -- anti-diagonal wavefront dynamic programs (DTW, Frechet,
// LCSS) for batches of query x candidate pairs.
//
// Layout of the work: a warp is split into segments of G lanes; each segment
// owns one pair.  The pair's rows (query points) are dealt to the segment in
// rounds of G*R rows: lane l of the segment holds rows l*R .. l*R+R-1 of the
// round in registers.  Inside a round the lanes run a skewed wavefront: at
// step s lane l computes column j = lo + s - l of all its R rows, so the
// value it needs from the row above (the bottom row of lane l-1) was produced
// one step earlier and arrives by __shfl_up_sync.  Lane G-1 also writes its
// bottom row to a per-segment shared-memory row buffer, which lane 0 reads as
// "the row above" in the next round.  The column range of a round is
// restricted to the band of its rows, cells outside a row's band are masked.
//
// Every pair's DP visits the same cells and performs the same FP32 operations
// whatever G and R are, so results do not depend on the launch shape.
//
// Reference kernels these replace: dtw_refine_kernel (CudaRuntime1/dtw.cu:41-96),
// lcss_refine_kernel_m_1 (lcss.cu:46-111), frechet_refine_kernel_m
// (frechet.cu:44-117): one CTA per pair, one barrier per anti-diagonal, every
// point re-read from global memory per cell.
#include "debug_bounds.cuh"
#include "dp_policies.cuh"

namespace tsim {
namespace {
using namespace dp;

constexpr int kDpThreads = 128;
constexpr int kNoColumn = 1 << 30;

template <class P, int G, int R>
__global__ void __launch_bounds__(kDpThreads) dp_pairs_kernel(DpArgs a) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char dp_smem[];
  constexpr int SEGS = 32 / G;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int sl = lane % G;  // lane within the segment
  const int seg = lane / G;
  V* buf = reinterpret_cast<V*>(dp_smem) + (size_t)(wib * SEGS + seg) * a.buf_len;
  const int warps_per_block = blockDim.x >> 5;
  const int gw = blockIdx.x * warps_per_block + wib;
  const int nw = gridDim.x * warps_per_block;

  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;
  for (int base = gw * SEGS; base < npairs; base += nw * SEGS) {
    const int wid = base + seg;
    const int pid = (wid < npairs && a.order) ? a.order[wid] : wid;
    const bool has = wid < npairs && a.pairs[pid].y >= 0;
    int n = 0, m = 0, q = 0;
    const float2* A = a.qpts;
    const float2* B = a.cpts;
    float thr = TSIM_INF;
    float aux = a.eps;  // the cell policy's parameter: eps, or the pair's aux value
    if (has) {
      int2 pr = a.pairs[pid];
      q = pr.x;
      if (pr.y < 0) {  // empty slot of a fixed-capacity pair list
        q = 0;
        pr.y = 0;
      }
      int64_t qo = a.qoff[q], co = a.coff[pr.y];
      n = (int)(a.qoff[q + 1] - qo);
      m = (int)(a.coff[pr.y + 1] - co);
      A += qo;
      B += co;
      if (a.thr) thr = a.thr[q];
      if (a.aux) aux = (float)a.aux[pid];
    }
    const int w = band_w(n, m, a.band_pct);
    const int rrow = result_row<P>(n, m, a.delta);
    const int rounds = has ? (n + G * R - 1) / (G * R) : 0;
    const int maxr = __reduce_max_sync(0xffffffffu, (unsigned)rounds);
    bool alive = has;
    V result = P::border();
    bool holds_result = false;
    long long cells = 0;  // band cells this lane computed for the pair
    // default result (pairs with an empty trajectory compute nothing); the
    // lane that captures the real value writes after this in program order
    if (has && sl == 0) store_result(a, pid, P::border());
    int prev_lo = 0, prev_hi = -1;

    for (int r = 0; r < maxr; ++r) {
      const bool act = alive && r < rounds;
      const int row0 = r * G * R + sl * R;
      float qx[R], qy[R];
      int jlo[R], jhi[R];
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = row0 + k;
        if (act && i < n) {
          float2 p = A[i];
          qx[k] = p.x;
          qy[k] = p.y;
          RowBand<P>::get(i, n, m, w, a.delta, jlo[k], jhi[k]);
          if (jhi[k] < jlo[k]) jlo[k] = jhi[k] = kNoColumn;
        } else {
          qx[k] = qy[k] = 0.0f;
          jlo[k] = jhi[k] = kNoColumn;  // empty row: no column is inside
        }
      }
      // column range of the round: band of its first and last rows
      int rlo = 0, rhi = -1;
      if (act) {
        int first = r * G * R, last = min(n - 1, (r + 1) * G * R - 1), t0, t1;
        RowBand<P>::get(first, n, m, w, a.delta, rlo, t0);
        RowBand<P>::get(last, n, m, w, a.delta, t1, rhi);
      }
      const int S = (act && rhi >= rlo) ? (rhi - rlo + G) : 0;
      const int Smax = (int)__reduce_max_sync(0xffffffffu, (unsigned)S);

      V left[R];
#pragma unroll
      for (int k = 0; k < R; ++k) left[k] = P::border();
      V outv = P::border();
      V prev_up = P::border();
      if (sl == 0 && act) {
        if (r == 0)
          prev_up = P::origin();
        else {
          int x = rlo - 1;
          prev_up = (x >= prev_lo && x <= prev_hi) ? buf[TSIM_SIDX(x, a.buf_len)] : P::border();
        }
      }
      float bmin = TSIM_INF;
      if (act && a.cells) {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (jlo[k] != kNoColumn) cells += jhi[k] - jlo[k] + 1;
      }

      for (int s = 0; s < Smax; ++s) {
        const int j = rlo + s - sl;
        V up = shfl_up_seg(outv, G);
        if (sl == 0) up = (r > 0 && j >= prev_lo && j <= prev_hi) ? buf[TSIM_SIDX(j, a.buf_len)] : P::border();
        const V diag = prev_up;
        prev_up = up;
        if (s < S && j >= rlo && j <= rhi) {
          const float2 cp = __ldg(B + j);
          V u = up, dg = diag;
#pragma unroll
          for (int k = 0; k < R; ++k) {
            const V lf = left[k];
            V v = P::cell(qx[k], qy[k], cp.x, cp.y, u, lf, dg, aux);
            const bool in = (unsigned)(j - jlo[k]) <= (unsigned)(jhi[k] - jlo[k]);
            v = in ? v : P::masked(lf);
            dg = lf;
            u = v;
            left[k] = v;
          }
          outv = u;
          if (sl == G - 1) buf[TSIM_SIDX(j, a.buf_len)] = outv;
          if (P::kMin) bmin = fminf(bmin, vf(outv));
        }
      }
      __syncwarp();
      if (act) {
#pragma unroll
        for (int k = 0; k < R; ++k)
          if (row0 + k == rrow) {
            result = left[k];
            holds_result = true;
          }
      }
      // lower bound of the pair: every warping path crosses every row, and
      // values never decrease along a path, so D >= min over any row.
      if (P::kMin && a.thr) {
        float lb = (act && row0 + R - 1 < n) ? bmin : 0.0f;
        lb = seg_max(lb, G);
        if (act && lb > thr) alive = false;
      }
      if (act) {
        int l0, h0;
        RowBand<P>::get(min(n - 1, (r + 1) * G * R - 1), n, m, w, a.delta, l0, h0);
        prev_lo = l0;
        prev_hi = h0;
      }
    }
    if (a.cells) {
      for (int o = G >> 1; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o, G);
      if (has && sl == 0) atomicAdd(a.cells, (unsigned long long)cells);
    }
    if (has && holds_result) store_result(a, pid, alive ? result : P::border());
    if (has && !alive && sl == 0) store_result(a, pid, P::border());
    __syncwarp();
  }
}

template <class P, int G, int R>
int launch_one(tsim_ctx* ctx, const DpArgs& a) {
  if (a.npairs <= 0) return TSIM_OK;
  constexpr int SEGS = 32 / G;
  const int warps = kDpThreads / 32;
  size_t smem = (size_t)warps * SEGS * a.buf_len * sizeof(typename P::V);
  auto kern = dp_pairs_kernel<P, G, R>;
  if (smem > 48 * 1024) TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kDpThreads, smem));
  if (per_sm < 1) return fail(TSIM_ERR_UNSUPPORTED, "dp kernel does not fit on an SM (candidate too long)");
  long long groups = (a.npairs + SEGS - 1) / SEGS;
  long long blocks_needed = (groups + warps - 1) / warps;
  long long blocks = std::min<long long>(blocks_needed, (long long)per_sm * ctx->num_sms);
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kDpThreads, smem, ctx->stream>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

template <class P, int G>
int launch_r(tsim_ctx* ctx, int R, const DpArgs& a) {
  switch (R) {
    case 1: return launch_one<P, G, 1>(ctx, a);
    case 2: return launch_one<P, G, 2>(ctx, a);
    case 4: return launch_one<P, G, 4>(ctx, a);
    default: return launch_one<P, G, 8>(ctx, a);
  }
}

template <class P>
int launch_g(tsim_ctx* ctx, int G, int R, const DpArgs& a) {
  switch (G) {
    case 4: return launch_r<P, 4>(ctx, R, a);
    case 8: return launch_r<P, 8>(ctx, R, a);
    case 16: return launch_r<P, 16>(ctx, R, a);
    default: return launch_r<P, 32>(ctx, R, a);
  }
}

// the FP64 re-score runs few pairs: two segment widths are enough
template <class P>
int launch_g64(tsim_ctx* ctx, int G, int R, const DpArgs& a) {
  return G <= 8 ? launch_r<P, 8>(ctx, R, a) : launch_r<P, 32>(ctx, R, a);
}

}  // namespace

int launch_dp(tsim_ctx* ctx, int kind, int G, int R, const DpArgs& a_in, int max_m) {
  DpArgs a = a_in;
  a.buf_len = (max_m + 4) & ~3;
  // fewer segments per warp when the row buffers would not fit in shared memory
  const size_t vbytes = (kind >= DP_DTW_SQ64) ? 8 : 4;  // FP64 and (hi, lo) kinds
  while (G < 32 && (size_t)(kDpThreads / 32) * (32 / G) * a.buf_len * vbytes > 200 * 1024) G *= 2;
  if ((size_t)(kDpThreads / 32) * (32 / G) * a.buf_len * vbytes > 200 * 1024)
    return fail(TSIM_ERR_UNSUPPORTED, "candidate trajectory too long for the shared-memory row buffer");
  switch (kind) {
    case DP_DTW_REF: return launch_g<PolDtwRef>(ctx, G, R, a);
    case DP_FRECHET_REF: return launch_g<PolFrechetRef>(ctx, G, R, a);
    case DP_LCSS: return launch_g<PolLcss>(ctx, G, R, a);
    case DP_DTW_SQ: return launch_g<PolDtwSq>(ctx, G, R, a);
    case DP_DTW_EU: return launch_g<PolDtwEu>(ctx, G, R, a);
    case DP_FRECHET_SQ: return launch_g<PolFrechetSq>(ctx, G, R, a);
    case DP_DTW_SQ64: return launch_g64<PolDtwSq64>(ctx, G, R, a);
    case DP_DTW_EU64: return launch_g64<PolDtwEu64>(ctx, G, R, a);
    case DP_FRECHET_SQ64: return launch_g64<PolFrechetSq64>(ctx, G, R, a);
    case DP_DTW_SQC: return launch_g64<PolDtwSqC>(ctx, G, R, a);
    case DP_DTW_EUC: return launch_g64<PolDtwEuC>(ctx, G, R, a);
    case DP_FRECHET_SQC: return launch_g64<PolFrechetSqC>(ctx, G, R, a);
    case DP_FRECHET_WIN: return launch_g64<PolFrechetWin>(ctx, G, R, a);
  }
  return fail(TSIM_ERR_INVALID_ARG, "unknown dp kind");
}

// Launch shape: the band of one row spans about `width` columns and moves
// `slope` columns per row; a round of G*R rows costs (width + (G*R-1)*slope +
// G - 1) steps of R cells per lane for G*R*width useful cells.  Pick the
// (G, R) with the best useful/issued ratio, preferring fewer segments per
// warp on ties (less work left idle when a warp's pairs differ in length).
void dp_shape(int kind, int n, int m, int wd, int& G, int& R) {
  double width, slope = n > 1 ? double(m - 1) / double(n - 1) : 0.0;
  if (wd < 0) {
    width = m;
    slope = 0.0;
  } else if (kind == DP_LCSS) {
    width = std::min<double>(m, 2.0 * wd + 1.0);
    slope = 1.0;
  } else {
    int lo, hi;
    band_row(n / 2, n, m, wd, lo, hi);
    width = hi - lo + 1;
  }
  double best = -1.0;
  G = 32;
  R = 1;
  const int Gs[4] = {32, 16, 8, 4};
  const int Rs[4] = {1, 2, 4, 8};
  for (int gi = 0; gi < 4; ++gi)
    for (int ri = 0; ri < 4; ++ri) {
      int g = Gs[gi], r = Rs[ri];
      int rows = g * r;
      int rounds = (n + rows - 1) / rows;
      double steps_per_round = std::min<double>(m, width + (rows - 1) * slope) + g - 1;
      double issued = rounds * steps_per_round * rows;  // lane-cells
      double useful = double(n) * width;
      // per-step overhead (shuffle, buffer, load, loop) amortised over R cells
      double cost = issued * (1.0 + 6.0 / (7.0 * r)) + rounds * rows * 20.0;
      double score = useful / cost;
      if (score > best * 1.03) {
        best = score;
        G = g;
        R = r;
      }
    }
}

}  // namespace tsim
