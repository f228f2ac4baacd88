// dp_diag.cu -- anti-diagonal wavefront DP for banded / windowed pairs.
//
// One warp per (query, candidate) pair (or 2 or 8 warps, for the
// latency-bound rounds).  Cell (i, j) is computed at step t = i + j.  Rows
// are dealt to lanes in groups of R consecutive rows, round robin: lane l
// owns rows R*(l + 32k) .. R*(l + 32k) + R - 1 for k = 0, 1, ...  At step t a
// lane computes column t - i of each row i of its current group, so all R
// cells of a step depend only on the previous step: the row above a group
// (the last row of the previous lane's group) arrives by one register
// shuffle (across warps, through shared memory behind a barrier), and there
// is no row buffer and no per-round skew -- the critical path of a pair is
// its n + m - 1 anti-diagonals.
//
// A lane moves to its next group when that group's first cell comes up.
// This is valid when a group has finished -- and the next lane has consumed
// its last row -- before the lane's next group starts.  With the band
// |i(m-1) - j(n-1)| <= W (W = w (min(n,m)-1)) that holds whenever
// 2W < 31 R (n + m - 2); for a full row (no band) when m <= 31 R + 1; for
// an LCSS window |i - j| <= delta when delta <= 31 R (32 W lanes: 32 W - 1
// in place of 31).  Pairs that fail the condition are listed for the next
// pass, the last one for the round-striped kernel (dp_kernels.cu).
//
// A lane's band columns come from integer ramps stepped by additions; its
// next group (band bases and widths, query points, the first candidate
// point) is prepared ahead for all lanes at once on every 16th step, so a
// switch is register moves; the candidate point of the next step is loaded
// one step ahead from the pair's copy in shared memory (through L1 for
// candidates too long to stage).  The step loop runs two steps per
// iteration.  Multi-warp pairs are claimed dynamically from a counter.
//
// Early abandon: every warping path crosses one of any two consecutive
// anti-diagonals and DP values never decrease along a path, so the minimum
// over the last two anti-diagonals bounds the final value from below; DTW's
// survivor round adds the LB_Keogh terms of the columns still ahead.
#include <type_traits>
#include <vector>

#include "bounds.cuh"
#include "debug_bounds.cuh"
#include "dp_policies.cuh"
#include "dp_ramps.cuh"

namespace tsim {
namespace {
using namespace dp;

constexpr int kDiagThreads = 128;
constexpr int kMaxStagedCols = 768;      // candidate points staged per warp (6 KiB)
constexpr int kCtaWarps = 8;             // warps of a CTA-per-pair launch
constexpr int kMaxStagedColsCta = 4096;  // candidate points staged per CTA (32 KiB)
constexpr int kNone = 1 << 30;

}  // namespace

__host__ __device__ bool diag_ok(bool lcss, int n, int m, int wd, int R, int lanes) {
  if (n < 2 || m < 2) return false;
  const long long span = (long long)(lanes - 1) * R;  // rows between a lane's groups, less one group
  if (wd < 0) return m <= span + 1;
  if (lcss) return wd <= span;
  const long long W = (long long)wd * ((n < m ? n : m) - 1);
  return 2 * W < span * (n + m - 2);
}

namespace {

// DTW on a warp per pair, abandoning against thresholds with the queries'
// sparse tables at hand: each pair's columns get a lower bound (the distance
// from the candidate point to the box of the query rows its band admits),
// whose suffix sums are kept in shared memory next to the staged candidate.
// (queries of up to 16,384 points: the per-check sums take (max_n + col_cap)
// / 16 floats of shared memory per pair)
template <class P, int W>
__host__ __device__ bool diag_suffix(const DpArgs& a) {
  return W == 1 && (std::is_same<P, PolDtwSq>::value || std::is_same<P, PolDtwEu>::value) &&
         a.qtab != nullptr && a.thr != nullptr && a.max_n > 0 && a.max_n <= 16384;
}

// abandon checks (every 16 steps) of a pair of up to max_n x col_cap points
__host__ __device__ inline int diag_checks(int max_n, int col_cap) {
  return (max_n + col_cap) / 16 + 2;
}

// resident CTAs per SM asked of the register allocator.  FP32 R <= 2: 7
// (28 warps, 72 registers): at 8 CTAs (64 registers) the allocator spilled
// 44 to 60 bytes in the step loop depending on the argument struct's layout,
// and the survivor launch's tail leaves about 30 % of the warps active
// anyway.  Fewer for the compensated (two-float) values and for R = 4.
template <class P, int R>
constexpr int diag_min_blocks() {
  return R >= 8                             ? 1  // long unbanded rows: latency, not occupancy
         : sizeof(typename P::V) > 4        ? (R == 1 ? 8 : (R == 2 ? 6 : 4))
         : std::is_same<P, PolDtwEu>::value ? (R == 1 ? 8 : (R == 2 ? 6 : 4))
                                            : (R <= 2 ? 7 : 5);
}

// W warps per pair: 1 (a warp per pair, kDiagThreads per CTA) or kCtaWarps
// (a CTA per pair: its 32 W lanes share the rows, the row above a warp's
// first lane crosses warps through shared memory once per step)
template <class P, int R, int W>
__global__ void __launch_bounds__(W == 1 ? kDiagThreads : 32 * W,
                                  (W == 1 ? diag_min_blocks<P, R>() : 1))
    dp_diag_kernel(DpArgs a, int col_cap, int* spill, int* nspill) {
  using V = typename P::V;
  extern __shared__ __align__(16) float2 diag_cand[];
  __shared__ V xbuf[2][W];  // W > 1: last lane's value of each warp, by step parity
  __shared__ float xred[W];  // W > 1: each warp's abandon bound
  constexpr bool kLcss = !P::kMin;
  constexpr int kLanes = 32 * W;     // lanes per pair
  constexpr int kRound = kLanes * R;  // rows between two groups of one lane
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int pl = W == 1 ? lane : (int)threadIdx.x;  // lane within the pair
  const int slot = W == 1 ? (blockIdx.x * blockDim.x + threadIdx.x) >> 5 : blockIdx.x;
  const int nslots = W == 1 ? (gridDim.x * blockDim.x) >> 5 : gridDim.x;
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;
  float2* cs = diag_cand + (W == 1 ? (size_t)warp * col_cap : 0);  // this pair's candidate

  // Work items.  A warp per pair strides over the pairs (sorted longest
  // first).  Two warps or a CTA per pair (latency rounds, whose lists hold
  // padding entries: a query's re-score slots beyond its set) take their
  // first pair by slot, then the next unclaimed one from the launch's counter
  // (nspill[1], zeroed with the spill count): a static stride could hand one
  // CTA two real pairs and double the round's latency (re-score stage 0.25
  // -> 0.19 ms).  For a warp per pair the claim's round trip cost more than
  // the shorter tail saved.
  __shared__ int next_item;
  auto fetch = [&](int wk) -> int {
    if (W == 1 || nspill == nullptr) return wk + nslots;
    if (threadIdx.x == 0) next_item = nslots + atomicAdd(nspill + 1, 1);
    __syncthreads();
    const int v = next_item;
    __syncthreads();
    return v;
  };
  for (int wk = slot; wk < npairs; wk = fetch(wk)) {
    const int pid = a.order ? a.order[wk] : wk;
    const int2 pr = a.pairs[pid];
    if (pr.y < 0) continue;
    const int q = pr.x;
    const int64_t qo = a.qoff[q], co = a.coff[pr.y];
    const int n = (int)(a.qoff[q + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    const float2* A = a.qpts + qo;
    const float2* B = a.cpts + co;
    // the candidate's points, read once into shared memory when they fit
    // (longer candidates are read through L1 step by step)
    const bool staged = m <= col_cap;
    const int w = band_w(n, m, a.band_pct);
    const int wd = kLcss ? a.delta : w;
    if (!diag_ok(kLcss, n, m, wd, R, kLanes)) {
      if (pl == 0 && spill) spill[atomicAdd(nspill, 1)] = pid;
      continue;
    }
    const float thr = a.thr ? a.thr[q] : TSIM_INF;
    // the cell policy's parameter: eps, or the pair's aux value (the exact
    // Frechet window's FP32 value)
    const float aux = a.aux ? (float)a.aux[pid] : a.eps;
    const int rrow = result_row<P>(n, m, a.delta);
    if (pl == 0) store_result(a, pid, P::border());

    if (W == 1) {
      __syncwarp();
      if (staged)
        for (int j = lane; j < m; j += 32) cs[TSIM_SIDX(j, col_cap)] = __ldg(B + j);
      __syncwarp();
    } else {
      __syncthreads();  // the previous pair is done with the staging and the exchange
      if (staged)
        for (int j = pl; j < m; j += kLanes) cs[TSIM_SIDX(j, col_cap)] = __ldg(B + j);
      if (lane == 31) xbuf[0][warp] = xbuf[1][warp] = P::border();
      __syncthreads();
    }
    const float2* C = staged ? cs : B;
    // candidate point of column j; columns outside 0 .. m-1 (cells outside
    // the band, whose values are masked) read point m-1
    auto cand = [&](int j) -> float2 { return C[min((unsigned)j, (unsigned)(m - 1))]; };

    // Remaining-columns bound (DTW, warp per pair): every path crosses every
    // column after the one where it crosses anti-diagonals t-1, t, and a cell
    // of column j costs at least the distance from candidate point j to the
    // box of the query rows j's band admits.  sfx[j] = sum of those bounds
    // over columns j .. m-1 (rounded down; sfx[m] = 0), built once per pair;
    // chk[c] = the part of it the abandon check at step 16c + 15 adds (the
    // columns after the last one of anti-diagonals 16c + 14 and 16c + 15).
    // The FP32 path sum that adds those columns' costs can round below their
    // exact sum by at most (n+m+8) 2^-24 relative, so the check compares with
    // the threshold divided by 1 minus that.
    const int sfx_cap = col_cap + 1, chk_cap = diag_checks(a.max_n, col_cap);
    float* sfx = reinterpret_cast<float*>(diag_cand + (size_t)(blockDim.x >> 5) * col_cap) +
                 (size_t)warp * (sfx_cap + chk_cap);
    float* chk = sfx + sfx_cap;
    const int t_last = n + m - 2;
    const bool suffix = diag_suffix<P, W>(a) && staged && n <= a.max_n &&
                        (t_last >> 4) < chk_cap;
    float thr_chk = thr;  // threshold of the abandon check
    if (suffix) {
      const long long wband = w >= 0 ? (long long)w * (min(n, m) - 1) : -1;
      const QTable T = qtable_view(a.qtab + (size_t)q * qtable_stride(a.max_n), n);
      float carry = 0.0f;  // bound of the columns after the current block
      for (int b0 = ((m - 1) >> 5) << 5; b0 >= 0; b0 -= 32) {  // blocks of 32 columns, last first
        const int j = b0 + lane;
        float v = 0.0f;
        if (j < m) {
          int lo = 0, hi = n - 1;
          if (wband >= 0) {
            lo = max(0, floordiv_i((long long)j * (n - 1) - wband + (m - 2), m - 1));  // ceil
            hi = min(n - 1, floordiv_i((long long)j * (n - 1) + wband, m - 1));
          }
          if (lo <= hi) {
            const float4 bx = qtable_box(T, lo, hi);
            const float2 c = cs[TSIM_SIDX(j, col_cap)];
            v = box_pt_d2_rd(bx.x, bx.y, bx.z, bx.w, c.x, c.y);
            if (std::is_same<P, PolDtwEu>::value) v = __fsqrt_rd(v);
          } else {
            v = TSIM_INF;  // a column with no admissible row: no path
          }
        }
        // suffix sums inside the block (lane l: columns j .. b0 + 31), then
        // the columns after it
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float u = __shfl_down_sync(0xffffffffu, v, o);
          if (lane + o < 32) v = __fadd_rd(v, u);
        }
        v = __fadd_rd(v, carry);
        if (j < m) sfx[TSIM_SIDX(j, sfx_cap)] = v;
        carry = __shfl_sync(0xffffffffu, v, 0);
      }
      if (lane == 0) sfx[TSIM_SIDX(m, sfx_cap)] = 0.0f;
      __syncwarp();
      for (int c = lane; c <= (t_last >> 4); c += 32) {
        const int t = 16 * c + 15;  // the largest column of anti-diagonals t-1, t
        int jmax = min(t, m - 1);
        if (wband >= 0) jmax = min(jmax, floordiv_i((long long)t * (m - 1) + wband, n + m - 2));
        chk[TSIM_SIDX(c, chk_cap)] = sfx[TSIM_SIDX(jmax + 1, sfx_cap)];
      }
      __syncwarp();
      const float shrink = __fsub_rd(1.0f, __fmul_ru((float)(n + m + 8), 6.03e-8f));
      thr_chk = __fdiv_ru(thr, shrink);
    }

    const Ramps rp = make_ramps(n, m, wd, kLcss);
    const int row_q = (int)(rp.a / rp.d), row_r = (int)(rp.a % rp.d);
    const int rnd_q = (int)(kRound * rp.a / rp.d), rnd_r = (int)(kRound * rp.a % rp.d);

    // The lane's current group (first row i0) and its next one (first row
    // i1, starting at step ns), prepared ahead: a switch is register moves
    // only.  Lanes switch at different steps, so whatever a switch executes
    // the warp issues once per lane; the preparation (band ramps, point
    // loads) instead runs for every lane that needs it at once, on every
    // 16th step -- a lane's switches are at least 32 R W steps apart.
    int i1 = R * pl;
    Ramp L1 = rp.lo_at(i1), H1 = rp.hi_at(i1);  // band ramps at row i1
    float nqx[R], nqy[R];
    int nbase[R];
    unsigned nwdt[R];
    int ns;  // step of the next group's first cell (-1: not prepared yet)
    float2 ncand;
    auto prepare = [&]() {
      Ramp L = L1, H = H1;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int lo = rp.lo(L), hi = rp.hi(H);
        const bool ok = i1 + r < n && hi >= lo;
        nbase[r] = ok ? i1 + r + lo : 0x3fffffff;
        nwdt[r] = ok ? (unsigned)(hi - lo) : 0u;
        const float2 p = i1 + r < n ? __ldg(A + i1 + r) : make_float2(0.f, 0.f);
        nqx[r] = p.x;
        nqy[r] = p.y;
        if (r + 1 < R) {
          rp.step(L, row_q, row_r);
          rp.step(H, row_q, row_r);
        }
      }
      const int lo = rp.lo(L1), hi = rp.hi(H1);
      ns = i1 < n && hi >= lo ? i1 + lo : 0x7fffffff;  // its first cell's step
      ncand = cand(lo);                                 // and column
    };
    int i0 = 0;
    float qx[R], qy[R];
    int base[R];      // step at which row r's band starts: t - base = column - lo
    unsigned wdt[R];  // band width - 1 (empty rows: never in band)
    V left[R], left2[R];  // each row's values one and two columns back
    auto take_next = [&]() {
      i0 = i1;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        base[r] = nbase[r];
        wdt[r] = nwdt[r];
        qx[r] = nqx[r];
        qy[r] = nqy[r];
        left[r] = left2[r] = P::border();
      }
      ns = -1;  // until the next preparation
    };
    auto advance = [&]() {
      i1 += kRound;
      rp.step(L1, rnd_q, rnd_r);
      rp.step(H1, rnd_q, rnd_r);
      prepare();
    };
    prepare();
    take_next();
    advance();
    // lane 0's first group holds row 0, whose row above is the virtual row -1
    // (+inf, with D(-1,-1) = origin)
    bool first = pl == 0;
    V out = P::border();
    V prev_raw = P::border();  // the shuffled value of the previous step
    V dg0 = P::origin();       // D(-1,-1), read once
    float2 cw[R];
#pragma unroll
    for (int r = 0; r < R; ++r) cw[r] = make_float2(0.f, 0.f);
    // candidate point of the next step, loaded one step ahead (at a switch,
    // the prepared group's first column)
    float2 cnext = cand(-i0);
    V result = P::border();
    bool holds = false;
    bool alive = true;
    float mprev = TSIM_INF;
    const bool check = P::kMin && a.thr != nullptr;
    const int t_end = n + m - 2;
    int t_ab = t_end;

    // two steps per loop iteration: the registers of the rows' values one and
    // two columns back and of the candidate points alternate between the two
    // halves instead of being copied every step
#pragma unroll 2
    for (int t = 0; t <= t_end; ++t) {
      if (t == ns) {  // this lane's next group starts now
        if ((unsigned)(rrow - i0) < (unsigned)R) {  // it holds the result row
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (i0 + r == rrow) {
              result = left[r];
              holds = true;
            }
        }
        take_next();
        first = false;
        cnext = ncand;
      }
      if ((t & 15) == 0 && ns < 0) advance();
      // the last row of the previous lane's group, one column back: the row
      // above this lane's first row
      V raw = shfl_lane(out, (lane + 31) & 31);
      if (W > 1 && lane == 0) raw = xbuf[(t + 1) & 1][(warp + W - 1) % W];  // the previous warp's
      const V up_in = first ? P::border() : raw;
      const V dg_in = first ? dg0 : prev_raw;
      dg0 = P::border();
      prev_raw = raw;
#pragma unroll
      for (int r = R - 1; r > 0; --r) cw[r] = cw[r - 1];
      cw[0] = cnext;
      cnext = cand(t + 1 - i0);
      // row r computes column t - i0 - r: its up neighbour is row r-1 one step
      // ago and its diagonal neighbour row r-1 two steps ago, so rows are
      // visited last to first before row r-1 is overwritten
#pragma unroll
      for (int r = R - 1; r >= 0; --r) {
        const V lf = left[r];
        const V up = r > 0 ? left[r > 0 ? r - 1 : 0] : up_in;
        const V dg = r > 0 ? left2[r > 0 ? r - 1 : 0] : dg_in;
        V v = P::cell(qx[r], qy[r], cw[r].x, cw[r].y, up, lf, dg, aux);
        const bool in = (unsigned)(t - base[r]) <= wdt[r];
        v = in ? v : P::masked(lf);
        left2[r] = lf;
        left[r] = v;
      }
      out = left[R - 1];
      if (check && (t & 15) >= 14) {
        // minimum of this anti-diagonal's cells, all R rows (masked cells are
        // +inf): three-operand mins, then a last two-operand one if needed;
        // taken on the last two steps of every 16
        float mstep = vf(left[0]);
        int r = 1;
#pragma unroll
        for (; r + 1 < R; r += 2) mstep = min3f(mstep, vf(left[r]), vf(left[r + 1]));
        if (r < R) mstep = fminf(mstep, vf(left[r < R ? r : 0]));
        const float prev = mprev;
        mprev = mstep;
        if ((t & 15) == 15) {
          const float two = fminf(mstep, prev);
          float lb = __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(two)));
          if (suffix) lb = __fadd_rd(lb, chk[TSIM_SIDX(t >> 4, chk_cap)]);  // plus the remaining columns
          if (W > 1) {  // over the pair's warps (reads after this step's barrier)
            if (lane == 0) xred[warp] = lb;
            if (lane == 31) xbuf[t & 1][warp] = out;
            __syncthreads();
#pragma unroll
            for (int w2 = 0; w2 < W; ++w2) lb = fminf(lb, xred[w2]);
          }
          if (lb > thr_chk) {  // uniform across the pair
            alive = false;
            t_ab = t;
            break;
          }
          if (W > 1) continue;  // this step's exchange and barrier are done
        }
      }
      if (W > 1) {  // hand the last lane's value to the next warp
        if (lane == 31) xbuf[t & 1][warp] = out;
        __syncthreads();
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (i0 + r == rrow) {
        result = left[r];
        holds = true;
      }
    if (a.cells) {  // cells of the anti-diagonals 0 .. t_ab inside the band
      const Ramps rp = make_ramps(n, m, kLcss ? a.delta : band_w(n, m, a.band_pct), kLcss);
      long long cells = 0;
      const int q32 = (int)(kLanes * rp.a / rp.d), r32 = (int)(kLanes * rp.a % rp.d);
      Ramp L = rp.lo_at(pl), H = rp.hi_at(pl);
      for (int i = pl; i < n; i += kLanes) {
        const int lo = rp.lo(L), hi = min(rp.hi(H), t_ab - i);
        if (hi >= lo) cells += hi - lo + 1;
        rp.step(L, q32, r32);
        rp.step(H, q32, r32);
      }
      for (int o = 16; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o);
      if (lane == 0) atomicAdd(a.cells, (unsigned long long)cells);
    }
    if (W == 1) __syncwarp(); else __syncthreads();
    if (holds) store_result(a, pid, alive ? result : P::border());
    if (!alive && pl == 0) store_result(a, pid, P::border());
    if (W == 1) __syncwarp(); else __syncthreads();
  }
}

template <class P, int R, int W>
int launch_diag_one(tsim_ctx* ctx, const DpArgs& a, int max_m, int* spill, int* nspill) {
  if (a.npairs <= 0) return TSIM_OK;
  const int threads = W == 1 ? kDiagThreads : 32 * W;
  const int pairs_per_cta = W == 1 ? kDiagThreads / 32 : 1;
  const int col_cap = (std::min(max_m, W == 1 ? kMaxStagedCols : kMaxStagedColsCta) + 1) & ~1;
  size_t smem = (size_t)pairs_per_cta * col_cap * sizeof(float2);
  if (diag_suffix<P, W>(a))
    smem += (size_t)pairs_per_cta * (col_cap + 1 + diag_checks(a.max_n, col_cap)) * sizeof(float);
  auto kern = dp_diag_kernel<P, R, W>;
  if (smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  long long blocks = std::min<long long>((a.npairs + pairs_per_cta - 1) / pairs_per_cta,
                                         (long long)std::max(per_sm, 1) * ctx->num_sms);
  kern<<<(unsigned)std::max(blocks, 1ll), threads, smem, ctx->stream>>>(a, col_cap, spill, nspill);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

template <class P, int W>
int launch_diag_r(tsim_ctx* ctx, int R, const DpArgs& a, int max_m, int* spill, int* nspill) {
  switch (R) {
    case 1: return launch_diag_one<P, 1, W>(ctx, a, max_m, spill, nspill);
    case 2: return launch_diag_one<P, 2, W>(ctx, a, max_m, spill, nspill);
    case 4: return launch_diag_one<P, 4, W>(ctx, a, max_m, spill, nspill);
    case 8:  // a warp, or a CTA of 8 warps (full rows of up to 2041 columns)
      if constexpr (W == 1 || W == kCtaWarps) return launch_diag_one<P, 8, W>(ctx, a, max_m, spill, nspill);
      break;
    default:
      if constexpr (W == 1) return launch_diag_one<P, 16, 1>(ctx, a, max_m, spill, nspill);
      break;
  }
  return fail(TSIM_ERR_UNSUPPORTED, "no CTA-per-pair kernel with this many rows per lane");
}

template <class P>
int launch_chain(tsim_ctx* ctx, int R0, int warps, const DpArgs& a, int max_m, int* spill,
                 int* nspill, int* tmp, int* ntmp, int rcap = 0) {
  // R0, 2 R0, .. Rmax: each pass takes the pairs the previous one spilled, so
  // every pair runs with the fewest rows per lane-group its shape admits
  // (fewer rows in flight, fewer masked cells); the last pass writes `spill`.
  // A warp per pair goes to R = 16 (full rows of up to 497 columns), two
  // warps per pair to R = 4 (253 columns), a CTA of eight to R = 8 (2041).
  // A pass takes every pair with both lengths >= 2 once the widest band
  // (any band width is at most that of the longest lengths, and
  // 2 (min(n,m) - 1) <= n + m - 2), the window or the longest full row fits
  // its lanes: the chain stops there, and only degenerate pairs are left for
  // the striped kernel.
  int rmax = warps == 1 ? 16 : (warps == kCtaWarps ? 8 : 4);
  if (rcap > 0) rmax = std::min(rmax, rcap);
  const int lanes = 32 * warps;
  auto takes_all = [&](int R) {
    if (a.max_n <= 0) return false;  // query lengths unknown
    const long long span = (long long)(lanes - 1) * R;
    const bool lcss = std::is_same<P, PolLcss>::value;
    const int wd = lcss ? a.delta : band_w(a.max_n, max_m, a.band_pct);
    if (wd < 0) return max_m <= span + 1;
    return wd < span;
  };
  std::vector<int> rs;
  for (int R = std::max(1, std::min(R0, rmax)); R <= rmax; R *= 2) {
    rs.push_back(R);
    if (takes_all(R)) break;
  }
  const int np = (int)rs.size();
  DpArgs in = a;
  for (int p = 0; p < np; ++p) {
    const bool to_spill = ((np - 1 - p) & 1) == 0;
    int* out = to_spill ? spill : tmp;
    int* nout = to_spill ? nspill : ntmp;
    TSIM_CUDA(cudaMemsetAsync(nout, 0, 2 * sizeof(int), ctx->stream));  // spills, work counter
    if (warps == 1)
      TSIM_TRY((launch_diag_r<P, 1>(ctx, rs[p], in, max_m, out, nout)));
    else if (warps == 2)
      TSIM_TRY((launch_diag_r<P, 2>(ctx, rs[p], in, max_m, out, nout)));
    else
      TSIM_TRY((launch_diag_r<P, kCtaWarps>(ctx, rs[p], in, max_m, out, nout)));
    in.order = out;
    in.npairs_dev = nout;
  }
  return TSIM_OK;
}

// the chain of launch_chain for a CTA per pair only (R = R0 .. 8)
template <class P>
int launch_chain_cta(tsim_ctx* ctx, int R0, const DpArgs& a, int max_m, int* spill, int* nspill,
                     int* tmp, int* ntmp) {
  std::vector<int> rs;
  for (int R = std::max(1, std::min(R0, 8)); R <= 8; R *= 2) {
    rs.push_back(R);
    if (a.max_n > 0 && max_m <= (kCtaWarps * 32 - 1) * R + 1) break;  // full rows: all fit
  }
  const int np = (int)rs.size();
  DpArgs in = a;
  for (int p = 0; p < np; ++p) {
    const bool to_spill = ((np - 1 - p) & 1) == 0;
    int* out = to_spill ? spill : tmp;
    int* nout = to_spill ? nspill : ntmp;
    TSIM_CUDA(cudaMemsetAsync(nout, 0, 2 * sizeof(int), ctx->stream));  // spills, work counter
    TSIM_TRY((launch_diag_r<P, kCtaWarps>(ctx, rs[p], in, max_m, out, nout)));
    in.order = out;
    in.npairs_dev = nout;
  }
  return TSIM_OK;
}

}  // namespace

int launch_dp_diag(tsim_ctx* ctx, int kind, int R, const DpArgs& a, int max_m, int* spill,
                   int* nspill, int* tmp, int* ntmp, int warps, int rmax) {
  const int W = warps > 2 ? kCtaWarps : warps;
  if (kind == DP_FRECHET_WIN) {
    // the exact FP64 Frechet re-score: few, possibly long full-row pairs
    // (latency), on a CTA per pair only
    if (W != kCtaWarps)
      return fail(TSIM_ERR_UNSUPPORTED, "the exact Frechet re-score runs on a CTA per pair");
    return launch_chain_cta<PolFrechetWin>(ctx, R, a, max_m, spill, nspill, tmp, ntmp);
  }
  switch (kind) {
    case DP_DTW_SQ: return launch_chain<PolDtwSq>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_DTW_EU: return launch_chain<PolDtwEu>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_LCSS: return launch_chain<PolLcss>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_FRECHET_SQ:
      return launch_chain<PolFrechetSq>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_DTW_SQC: return launch_chain<PolDtwSqC>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_DTW_EUC: return launch_chain<PolDtwEuC>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
    case DP_FRECHET_SQC:
      return launch_chain<PolFrechetSqC>(ctx, R, W, a, max_m, spill, nspill, tmp, ntmp, rmax);
  }
  return fail(TSIM_ERR_UNSUPPORTED, "no anti-diagonal kernel for this DP kind");
}

}  // namespace tsim
