// dp_lane.cu -- a lane per (query, candidate) pair: the throughput form of
// the FP32 DTW, discrete-Frechet and LCSS dynamic programs, for rounds with
// many more pairs than the GPU has warps.
//
// The warp-per-pair kernels (dp_diag.cu) spread one pair over many lanes, so
// a step's fixed work -- the shuffle that moves values between lanes, the
// band bookkeeping, the masking of lanes outside the band -- is shared by the
// few cells an anti-diagonal holds; with a 10 % band that costs about two warp
// instructions per cell.  Here a lane owns a whole pair and runs its matrix
// row block by row block:
//
//  - Orientation: the longer trajectory gives the rows ("outer"), the shorter
//    the columns ("inner"), so the band moves at most one column per row and
//    a row's band is at most 2w+1 columns wide.  DTW, Frechet and LCSS are
//    symmetric under this transpose (the band |i(m-1) - j(n-1)| <= W, the
//    window |i-j| <= delta and the cell costs are), and the minimum / maximum
//    of three values is exact in any order, so the values are the same bits
//    as the other kernels'.
//  - A pass takes R = 8 consecutive rows.  The lane sweeps the union of their
//    bands column by column, row k one column behind row k-1, so the R cells
//    of a step depend only on the last step's values: one inner point (read
//    through L1) and one value of the row above the pass (from shared
//    memory) enter per step, the R cells stay in registers, and the pass's
//    last row goes back to shared memory for the next pass.  Cells outside
//    their own row's band are masked as in the other kernels.
//  - The row above a pass lives in a ring of RING values per lane, slot
//    j mod RING, laid out [slot][thread] so that every lane reads and writes
//    its own bank.  A pair fits when the union of a pass's bands is at most
//    RING columns wide; pairs that do not fit (or that have fewer than two
//    points on a side) are listed in spill[] for the other kernels.
//  - Passes end on the last row: the first pass starts at row (no mod R) - R
//    when R does not divide the row count, its rows above row 0 being empty;
//    the empty row just above row 0 carries the origin D(-1,-1) to cell
//    (0, 0)'s diagonal.  The result is then the ring's value at the last
//    row's last band column.
//  - A lane moves on to its next pair on its own (items lane, lane + T, ...
//    of the launch's list, T the launch's lanes); the warp runs a pass as
//    long as the widest pass among its lanes.  Early abandon: every warping
//    path crosses every row, and values never decrease along a path, so when
//    the minimum of a pass's last row exceeds the query's threshold the pair
//    is dropped (result +inf), as in the other kernels.
//
// Reference kernels replaced: dtw_refine_kernel (CudaRuntime1/dtw.cu:41-96),
// lcss_refine_kernel_m_1 (lcss.cu:46-111) and frechet_refine_kernel_m
// (frechet.cu:44-117): a CTA per pair, every point re-read per cell and two
// barriers per anti-diagonal.
#include <type_traits>

#include "debug_bounds.cuh"
#include "dp_policies.cuh"
#include "dp_ramps.cuh"

namespace tsim {
namespace {
using namespace dp;

constexpr int kLaneThreads = 128;
constexpr int kLaneR = 8;          // rows per pass
constexpr int kEmptyLo = 1 << 30;  // an empty row's band start (no column is inside)

// the widest union of a pass's bands for a pair, bounded from its ramps
__device__ __forceinline__ int lane_union_bound(const Ramps& rp, int dq, int dr) {
  const long long width = (rp.Wl + rp.Wh) / rp.d + 2;
  const long long u = width + (long long)(kLaneR - 1) * (dq + (dr > 0 ? 1 : 0));
  return (int)(u < rp.m ? u : rp.m);
}

template <class P, int RING>
__global__ void __launch_bounds__(kLaneThreads, 3)
    dp_lane_kernel(DpArgs a, int* spill, int* nspill, int gate) {
  using V = typename P::V;
  static_assert(sizeof(V) == 4, "a ring slot holds a 4-byte value");
  static_assert((RING & (RING - 1)) == 0, "the ring size is a power of two");
  constexpr bool kLcss = !P::kMin;
  constexpr int R = kLaneR;
  extern __shared__ __align__(16) unsigned char lane_smem[];
  // slot s of this lane's ring: ring[RSLOT(s)]
  V* ring = reinterpret_cast<V*>(lane_smem);
#define RSLOT(s) TSIM_SIDX(((s) & (RING - 1)) * kLaneThreads + (int)threadIdx.x, RING * kLaneThreads)
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;
  const int T = gridDim.x * kLaneThreads;
  const bool check = P::kMin && a.thr != nullptr;
  int w = blockIdx.x * kLaneThreads + threadIdx.x;  // this lane's next work item
  if (npairs < gate) {
    // too few pairs to pay for a lane's latency: the whole list goes on, in
    // its order, to the warp-per-pair kernels
    for (int i = w; i < npairs; i += T) spill[i] = a.order ? a.order[i] : i;
    if (w == 0) *nspill = npairs;
    return;
  }

  // the lane's pair
  bool have = false;
  int pid = 0, no = 1, ni = 1, o0 = 0, pulo = 0, puhi = -1, dq = 0, dr = 0;
  const float2* O = a.qpts;
  const float2* I = a.qpts;
  float thr = TSIM_INF;
  Ramps rp{};
  Ramp rlo{0, 0}, rhi{0, 0};
  long long cells = 0;

  while (true) {
    // an idle lane claims its next pair
    while (!have && w < npairs) {
      const int id = a.order ? a.order[w] : w;
      w += T;
      const int2 pr = a.pairs[id];
      if (pr.y < 0) continue;  // empty slot of a fixed-capacity list
      const int64_t qo = a.qoff[pr.x], co = a.coff[pr.y];
      const int n = (int)(a.qoff[pr.x + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
      if (n < 2 || m < 2) {
        spill[atomicAdd(nspill, 1)] = id;
        continue;
      }
      const bool tr = n < m;  // rows on the longer trajectory
      O = tr ? a.cpts + co : a.qpts + qo;
      I = tr ? a.qpts + qo : a.cpts + co;
      no = tr ? m : n;
      ni = tr ? n : m;
      const int wd = kLcss ? a.delta : band_w(n, m, a.band_pct);
      rp = make_ramps(no, ni, wd, kLcss);
      dq = (int)(rp.a / rp.d);
      dr = (int)(rp.a % rp.d);
      if (lane_union_bound(rp, dq, dr) > RING) {
        spill[atomicAdd(nspill, 1)] = id;
        continue;
      }
      // LCSS with a window: rows past ni-1+delta are empty, and the result
      // is the last in-window value of row ni-1+delta
      if (kLcss && wd >= 0 && no > ni + wd) no = ni + wd;
      pid = id;
      thr = check ? a.thr[pr.x] : TSIM_INF;
      o0 = no % R == 0 ? 0 : no % R - R;
      rlo = rp.lo_at(0);
      rhi = rp.hi_at(0);
      pulo = 0;
      puhi = -1;
      have = true;
    }
    if (!__any_sync(0xffffffffu, have)) break;

    // the pass's rows: points, bands, and the union of the bands
    float2 o[R];  // the rows' points
    int base[R], span[R];  // row k is in its band at step s iff 0 <= s - base[k] <= span[k]
    int ulo = 0, uhi = -1;
    const int k0 = -o0;    // row 0's place in a first pass that starts above it
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int row = o0 + k;
      int l = kEmptyLo, h = kEmptyLo;
      float2 p = make_float2(0.0f, 0.0f);
      if (have && row >= 0) {
        l = rp.lo(rlo);
        h = rp.hi(rhi);
        rp.step(rlo, dq, dr);
        rp.step(rhi, dq, dr);
        p = __ldg(O + row);
        if (row == max(o0, 0)) ulo = l;
        uhi = h;
        cells += h - l + 1;
      } else if (P::kMin && have && row == -1) {
        // the empty row just above row 0 stands for the DTW / Frechet border
        // row: its point is the inner trajectory's first, so its cells at
        // the columns before 0 cost nothing and carry D(-1,-1) = origin from
        // its left value to row 0's diagonal at column 0
        p = __ldg(I);
        if (k0 >= 2) {
          l = 1 - k0;
          h = -1;
        }
      }
      o[k] = p;
      base[k] = l == kEmptyLo ? kEmptyLo : l + k;
      span[k] = l == kEmptyLo ? 0 : h - l;
    }
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (base[k] != kEmptyLo) base[k] -= ulo;
    const int S = have ? uhi - ulo + R : 0;  // steps: the union, then R-1 for the skew
    const int Smax = (int)__reduce_max_sync(0xffffffffu, (unsigned)S);

    // Row k works on column ulo + s - k at step s: its up neighbour (row k-1,
    // same column) is row k-1's value of the last step, its left one its own
    // value of the last step, its diagonal the up value it used then -- the
    // R cells of a step are independent.  Row 0's up values come from the
    // ring (the row above the pass).
    V L[R], U[R];
    float2 cw[R];  // inner point of each row's column
#pragma unroll
    for (int k = 0; k < R; ++k) {
      L[k] = (o0 + k == -1) ? P::origin() : P::border();
      U[k] = P::border();
      cw[k] = __ldg(I + min(max(ulo - k, 0), ni - 1));
    }
    if (o0 == 0)
      U[0] = P::origin();
    else if (o0 > 0 && ulo - 1 >= pulo && ulo - 1 <= puhi)
      U[0] = ring[RSLOT(ulo - 1)];
    int j0 = ulo;  // row 0's column
    V upv = j0 <= puhi ? ring[RSLOT(j0)] : P::border();
    float bmin = TSIM_INF;

    // One step: R cells, then row R-1's value to the ring.  MASK: test every
    // cell against its row's band (the steps where some row lies outside it).
    // Row R-1 reaches the union at step R-1; the ring slots of the earlier
    // steps' columns are not written (they may hold columns the pass reads).
    auto step = [&](const int s, auto mask_tag) {
      constexpr bool MASK = decltype(mask_tag)::value;
      const int jn = j0 + 1;  // the next step's inputs, ahead of this step's cells
      const float2 cpn = __ldg(I + min(jn, ni - 1));
      const V upn = ring[RSLOT(jn)];
#pragma unroll
      for (int k = R - 1; k >= 0; --k) {
        const V up = k > 0 ? L[k > 0 ? k - 1 : 0] : upv;
        const V lf = L[k];
        V v = P::cellp(o[k], cw[k], up, lf, U[k], a.eps);
        if (MASK) v = (unsigned)(s - base[k]) <= (unsigned)span[k] ? v : P::masked(lf);
        U[k] = up;
        L[k] = v;
      }
      if (!MASK || s >= R - 1) ring[RSLOT(j0 - (R - 1))] = L[R - 1];
      if (P::kMin) bmin = fminf(bmin, vf(L[R - 1]));
#pragma unroll
      for (int k = R - 1; k > 0; --k) cw[k] = cw[k - 1];
      cw[0] = cpn;
      upv = jn <= puhi ? upn : P::border();
      j0 = jn;
    };
#pragma unroll 8
    for (int s = 0; s < Smax; ++s) step(s, std::true_type{});

    if (have) {
      pulo = ulo;
      puhi = uhi;
      if (o0 + R >= no) {  // the last row: its last band column holds the result
        store_result(a, pid, ring[RSLOT(uhi)]);
        have = false;
      } else if (check && bmin > thr) {
        store_result(a, pid, P::border());
        have = false;
      } else {
        o0 += R;
      }
    }
  }
  if (a.cells) {
    for (int o = 16; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o);
    if ((threadIdx.x & 31) == 0 && cells) atomicAdd(a.cells, (unsigned long long)cells);
  }
}

#undef RSLOT

template <class P, int RING>
int launch_lane_one(tsim_ctx* ctx, const DpArgs& a, int* spill, int* nspill, int gate) {
  auto kern = dp_lane_kernel<P, RING>;
  const size_t smem = (size_t)RING * kLaneThreads * sizeof(typename P::V);
  if (smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLaneThreads, smem));
  const long long blocks = std::min<long long>((a.npairs + kLaneThreads - 1) / kLaneThreads,
                                               (long long)std::max(per_sm, 1) * ctx->num_sms);
  kern<<<(unsigned)std::max(blocks, 1ll), kLaneThreads, smem, ctx->stream>>>(a, spill, nspill, gate);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

template <class P>
int launch_lane_ring(tsim_ctx* ctx, const DpArgs& a, int ring, int* spill, int* nspill,
                     int gate) {
  return ring <= 64 ? launch_lane_one<P, 64>(ctx, a, spill, nspill, gate)
                    : launch_lane_one<P, 128>(ctx, a, spill, nspill, gate);
}

// ---- shape order of a pair list ---------------------------------------------
// Lanes of a warp run their passes in step, each as long as the widest among
// them, so a launch should hand neighbouring lanes pairs of one shape: a
// counting sort of the list by (longer length / 16, shorter length / 16),
// longest first.
constexpr int kShapeBuckets = 64 * 64;

__device__ __forceinline__ int lane_shape(const DpArgs& a, int id) {
  const int2 pr = a.pairs[id];
  if (pr.y < 0) return 0;
  const int n = (int)(a.qoff[pr.x + 1] - a.qoff[pr.x]), m = (int)(a.coff[pr.y + 1] - a.coff[pr.y]);
  const int hi = min(max(n, m) >> 4, 63), lo = min(min(n, m) >> 4, 63);
  return kShapeBuckets - 1 - (hi * 64 + lo);  // descending
}

__global__ void lane_hist_kernel(DpArgs a, int* cnt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npairs; i += gridDim.x * blockDim.x)
    atomicAdd(cnt + lane_shape(a, i), 1);
}

__global__ void __launch_bounds__(1024) lane_scan_kernel(int* cnt) {
  // exclusive prefix sum of kShapeBuckets counts, 4 per thread
  __shared__ int wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int4 c = reinterpret_cast<int4*>(cnt)[threadIdx.x];
  const int tot = c.x + c.y + c.z + c.w;
  int incl = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += v;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  int run = incl - tot + (warp > 0 ? wsum[warp - 1] : 0);
  int4 out;
  out.x = run;
  run += c.x;
  out.y = run;
  run += c.y;
  out.z = run;
  run += c.z;
  out.w = run;
  reinterpret_cast<int4*>(cnt)[threadIdx.x] = out;
}

__global__ void lane_scatter_kernel(DpArgs a, int* cnt, int* order) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npairs; i += gridDim.x * blockDim.x)
    order[atomicAdd(cnt + lane_shape(a, i), 1)] = i;
}
static_assert(kShapeBuckets == 1024 * 4, "the scan takes 4 buckets per thread of one block");

}  // namespace

int lane_sort(tsim_ctx* ctx, const DpArgs& a, int* order, int* counts) {
  if (a.npairs <= 0) return TSIM_OK;
  TSIM_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * kShapeBuckets, ctx->stream));
  const int blocks = (int)std::min<long long>((a.npairs + 255) / 256, 4ll * ctx->num_sms);
  lane_hist_kernel<<<blocks, 256, 0, ctx->stream>>>(a, counts);
  lane_scan_kernel<<<1, 1024, 0, ctx->stream>>>(counts);
  lane_scatter_kernel<<<blocks, 256, 0, ctx->stream>>>(a, counts, order);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx, 3);
  return TSIM_OK;
}
int lane_sort_buckets() { return kShapeBuckets; }

bool lane_kind(int kind) {
  return kind == DP_DTW_SQ || kind == DP_DTW_EU || kind == DP_FRECHET_SQ || kind == DP_LCSS;
}

// Pair count from which a survivor round runs faster on a lane per pair.
// A round takes about max(longest pair's latency, total cells / rate): a
// lane per pair has the longer latency (its cells one step of R at a time:
// about kLaneStepNs per step of its longest pair) and the higher rate.  The
// lane kernel wins once the warp-per-pair kernel's rate (kWarpCellsPerNs)
// needs longer for the round's cells than the lane kernel's latency, with
// pairs of half the longest lengths as the typical pair, and a factor 2 of
// margin for rounds that abandon early (shorter pairs favour the warp).
// Second condition, the tail: with every lane busy a lane runs about
// kLaneSatCellsPerNs / (lanes on the GPU) cells per ns, so a lane that draws
// the longest pair needs its cells / that, and the round on the warp kernels
// (kWaveCellsPerNs with their abandoning) must take twice as long.  Without
// it a 16-query DTW request of up to 2,048 points against the 1M serving
// database ran its 150 K survivors on lanes in 14.2 ms, on warps in 9.8 ms.
// DTW and Frechet only: their warp rounds run on the band-relative kernel;
// LCSS's run on the row-group kernel, whose rate the lanes keep beating.
int lane_gate_for(int kind, int max_n, int max_m, int band_pct, int delta, int num_sms) {
  constexpr double kLaneStepNs = 70.0, kWarpCellsPerNs = 435.0;  // 435 GCUPS
  constexpr double kLaneSatCellsPerNs = 1377.0, kWaveCellsPerNs = 700.0;
  auto cells = [&](int n, int m) {
    const int no = std::max(n, m), ni = std::min(n, m);
    const int wd = kind == DP_LCSS ? delta : (kind == DP_FRECHET_SQ ? -1 : band_w(n, m, band_pct));
    double width = ni;
    if (wd >= 0) width = kind == DP_LCSS ? std::min(ni, 2 * wd + 1)
                                         : std::min<double>(ni, 2.0 * wd * (ni - 1) / (no - 1) + 1);
    return std::max(1.0, (double)no * width);
  };
  const int no = std::max(max_n, max_m);
  const double width = cells(max_n, max_m) / no;
  const double latency_ns = std::ceil(no / (double)kLaneR) * (width + kLaneR) * kLaneStepNs;
  const double typical = cells(std::max(2, max_n / 2), std::max(2, max_m / 2));
  const double gate = 2.0 * latency_ns * kWarpCellsPerNs / typical;
  const double lanes = 3.0 * kLaneThreads * std::max(1, num_sms);  // 3 CTAs per SM
  const double longest_ns = cells(max_n, max_m) / (kLaneSatCellsPerNs / lanes);
  const double gate_tail = kind == DP_LCSS ? 0.0 : 2.0 * longest_ns * kWaveCellsPerNs / typical;
  return (int)std::min(std::max(gate, gate_tail), 1e9);
}

int lane_ring_for(int kind, int max_n, int max_m, int band_pct, int delta) {
  const int mn = std::min(max_n, max_m), mx = std::max(max_n, max_m);
  long long u;
  if (kind == DP_LCSS)
    u = delta < 0 ? mn : std::min<long long>(mn, 2ll * delta + 2 + (kLaneR - 1));
  else if (band_pct < 0 || kind == DP_FRECHET_SQ)
    u = mn;
  else  // the widest band of pairs up to these lengths: 2w + 1 columns, plus a pass's slope
    u = std::min<long long>(mn, 2ll * band_w(mx, mx, band_pct) + 2 + (kLaneR - 1));
  return u <= 64 ? 64 : 128;
}

int launch_dp_lane(tsim_ctx* ctx, int kind, const DpArgs& a, int ring, int* spill, int* nspill,
                   int gate) {
  TSIM_CUDA(cudaMemsetAsync(nspill, 0, sizeof(int), ctx->stream));
  if (a.npairs <= 0) return TSIM_OK;
  switch (kind) {
    case DP_DTW_SQ: return launch_lane_ring<PolDtwSq>(ctx, a, ring, spill, nspill, gate);
    case DP_DTW_EU: return launch_lane_ring<PolDtwEu>(ctx, a, ring, spill, nspill, gate);
    case DP_FRECHET_SQ: return launch_lane_ring<PolFrechetSq>(ctx, a, ring, spill, nspill, gate);
    case DP_LCSS: return launch_lane_ring<PolLcss>(ctx, a, ring, spill, nspill, gate);
  }
  return fail(TSIM_ERR_UNSUPPORTED, "no lane-per-pair kernel for this DP kind");
}

}  // namespace tsim
