// knn.cu -- exact k-nearest-neighbour search over a device-resident
// trajectory database for DTW, LCSS, discrete Frechet, symmetric Hausdorff
// and lock-step Euclidean.
//
// Stages (all on one stream, fixed launch shapes, data-dependent counts kept
// on the device so the whole sequence can be captured in a CUDA graph):
//   A  lb1_kernel      O(1) bound per (query, candidate) from 36-byte
//                      summaries (box, first and last point, length); each
//                      CTA also keeps its chunk's best few candidates; once
//                      B has set the threshold, compact_kernel lists the
//                      pairs the O(1) bound keeps and segfilter_kernel
//                      bounds them by 8 column segments per candidate and
//                      32 query row segments (a group of 8 lanes a pair);
//   B  seeds           the S best chunk candidates per query are refined
//                      exactly; the k-th best refined value, widened by the
//                      FP32 error bound, is the query's pruning threshold;
//   C  lb2_kernel      the listed pairs get the O(length) bound (banded
//                      LB_Keogh from the query's sparse table in global
//                      memory for DTW, its candidates fetched by bulk copy
//                      on databases larger than L2; box distances for
//                      Frechet and Hausdorff, the windowed eps-box count for
//                      LCSS; lock-step Euclidean passes the list on);
//   D  DP              round 1 (the best survivors by bound) tightens the
//                      threshold, then the remaining survivors run the
//                      wavefront DP (or the pairwise distance) with early
//                      abandon against it;
//   E  final           the k-th best FP32 value fixes the re-score set (all
//                      pairs within the FP32 error bound of it); the set is
//                      re-computed with compensated (hi, lo) FP32 arithmetic,
//                      pairs whose compensated values are within that
//                      tighter bound of a neighbour are re-computed in FP64
//                      with the oracle's arithmetic, and the set is sorted by
//                      (distance, candidate index).
// LCSS counts are exact integers in FP32, so LCSS skips the re-score.
//
// The reference's GPU path (CudaRuntime1/dtw.cu:99-234) instead ranks every
// candidate by a heuristic bound, refines a fixed 10 and returns one value:
// not an exact kNN.  This path returns the exact top-k ids and distances.
#include <cstring>
#include <type_traits>

#include "bounds.cuh"
#include "bulk_copy.cuh"
#include "topk.cuh"
#include "tsim_internal.cuh"

namespace tsim {

int summarize(tsim_ctx* ctx, const float2* pts, const int64_t* off, int count, float4* box,
              float4* ends, int* len);

namespace {

constexpr int kChunk = 256;     // candidates per stage-A CTA
constexpr int kSelThreads = 256;
constexpr int kSeg = 2048;       // list entries per CTA of the two-level selections
constexpr int kLb2Warps = 8;
constexpr int kGridWords = 4096;  // LCSS occupancy grid of a query: 131,072 cells (16 KiB)
constexpr int kQBlocks = 8;       // row blocks of a query in the O(1) bound

enum Meas { M_DTW = 0, M_LCSS = 1, M_FRECHET = 2, M_HAUSDORFF = 3, M_EUCLID = 4 };

// measures refined by the wavefront DP (the others by pairwise kernels)
constexpr bool is_dp(int meas) { return meas <= M_FRECHET; }
// re-score set ordered by compensated values (DTW: an FP32 path sum's error
// grows with the path); the others' FP32 value is one rounded cost (Frechet,
// Hausdorff) or a compensated sum (Euclidean) and is used as it is
constexpr bool compensated_rescore(int meas) { return meas == M_DTW; }
// values carried in the squared domain (sqrt applied to the reported distance)
constexpr bool is_squared(int meas) { return meas >= M_FRECHET; }

struct KArgs {
  // queries
  const float2* qpts;
  const int64_t* qoff;
  const float4* qbox;
  const float4* qends;
  const int* qlen;
  int nq;
  // database
  const float2* cpts;
  const int64_t* coff;
  const float4* cbox;
  const float4* cends;
  const int* clen;
  int C;
  int max_clen;
  int max_qlen;  // shared-memory tables are sized for this query length
  // parameters
  int k, S, T, nch;
  int plain;    // one DP pair per kernel launch (the unbatched comparison form)
  int brute;    // small request: every pair refined exactly, no bound stages
  int noprune;  // thresholds stay open: every pair is refined
  int cost;  // DTW: 0 squared, 1 Euclidean
  int band_pct;
  int delta;
  float eps;
  // scratch
  float* lb1;               // [nq*C]
  int* chunk_cand;          // [nq*nch*T]
  int2* seeds;              // [nq*S]
  unsigned* seedmap;        // [nq*Cw]
  int Cw;
  float* seed_vals;         // [nq*S]
  float* thr;               // [nq]  pruning / abandon threshold
  int* cnt0;                // [nq]  pairs the O(1) bound keeps (stage A, first half)
  int* cnt1;                // [nq]
  int* list1;               // [nq*C]
  int* cnt2;                // [nq]
  int* list2;               // [nq*C]  survivors of the O(length) bound
  float* lb2v;              // [nq*C]  their bound values
  int M;                    // round-1 pairs per query (best by O(length) bound)
  int2* r1pairs;            // [nq*M]
  float* r1vals;            // [nq*M]
  float* thr2;              // [nq]  threshold after round 1
  int* fcnt;                // [nq]  round-2 pairs per query (in list1)
  const float4* csegbox;    // [C*kSegs] candidate segment boxes
  const float2* csegsum;    // [C*kSegs] sums of the candidate segments' points
  float2* qpf;              // [nq*(max_qlen+1)] query prefix sums of p_j - p_0, FP32-rounded
  float* qpe;               // [nq] twice a bound on their FP64 accumulation error
  int lb2_cap;              // DTW O(length) stage: points per bulk-copy buffer (0: no bulk copies)
  int64_t ctotal;           // points in the database's array (bulk copies stay inside it)
  unsigned* status;         // device status word: bit 0 = a bounded wait ran out
  float4* qblk;             // [nq*kQBlocks] boxes of the query's row blocks
  int* spill;               // pairs the anti-diagonal kernel leaves to the striped one
  int* nspill;
  int* spill2;              // the list between passes of the anti-diagonal kernel
  int* nspill2;
  int* lanes;               // what the lane-per-pair kernel leaves to the warp-per-pair ones
  int* nlanes;
  int lane_gate;            // survivor rounds of at least this many pairs run a lane per
                            // pair (0: never)
  int lane_ring;            // its ring size (64 or 128)
  const float* thr_in;      // optional [nq]: a pruning threshold known beforehand (an earlier
                            //   identical query's), combined with the seeds' (else null)
  float* thr_out;           // optional [nq]: the final pruning threshold, for later requests
  int* waves;               // what the band-relative kernel leaves to the row-group ones
  int* nwaves;
  int wave;                 // DTW / Frechet rounds start on the band-relative kernel
  int rdiag;                // rows per lane-group of the anti-diagonal kernel (0: off)
  int rdiag_shape;          // the smallest R a warp per pair admits for the longest pair
  int rdiag_cta;            // the same for a CTA per pair (0: no R fits the longest pair)
  int rdiag_w2;             // the same for two warps per pair
  float4* qtab;             // [nq*tstride] query sparse tables (global memory)
  float4* qenv;             // LCSS with a window: [nq*env_stride] eps-inflated boxes of the
  int env_stride;           //   query rows [i-delta, i+delta], i < max_qlen+delta (else null)
  int tstride;
  int* off2;                // [nq+1]
  int* npairs;              // [1]
  int2* flat;               // [nq*C]
  int* order;               // [nq*C] shape-sorted schedule of flat
  int* shape_cnt;           // [kNumShapes]
  float* flat_vals;         // [nq*C]
  int nseg;                 // segments of kSeg entries per query (two-level selection)
  unsigned long long* segkeys;  // [nq*nseg*64] best keys of every segment
  unsigned long long* kthkey;   // [nq] key of the k-th best refined pair
  int* rraw;                    // [nq] pairs within the re-score bound (before the cap)
  int RC;
  int2* rpairs;             // [nq*RC] re-score set
  double* rdc;              // [nq*RC] compensated FP32 (hi+lo) values
  int2* r64pairs;           // [nq*RC] members of ambiguous clusters (else y = -1)
  double* r64;              // [nq*RC] FP64 values of those
  int* rcnt;                // [nq]
  int* n64;                 // [1] pairs sent to FP64
  int force64;              // re-score every pair in FP64 (bit-identical distances)
  // outputs
  int* ids;
  float* dists;
  double* dists64;
};

__device__ __forceinline__ double gamma_dp(int meas, int n, int m) {
  // relative error of an FP32 DP value against FP64 (both against exact):
  // every cost carries <= 4 roundings, a path of <= n+m-1 cells adds one
  // rounding per cell; Frechet values are single costs.
  const double u = 1.0 / 16777216.0;
  if (meas == M_FRECHET || meas == M_HAUSDORFF) return 8.0 * u;  // one FMA distance
  if (meas == M_EUCLID) return 16.0 * u;  // compensated sum of FMA terms
  return (double)(n + m + 8) * u * 1.01 + 1e-12;
}

// threshold widened by the error bound, rounded up to float
__device__ __forceinline__ float widen(float t, double g) {
  if (!(t < TSIM_INF)) return TSIM_INF;
  return __double2float_ru((double)t * (1.0 + g) / (1.0 - g) * (1.0 + 1e-12));
}

// ---------------------------------------------------------------------------
// stage A: O(1) bounds from summaries + chunk-local best candidates
// ---------------------------------------------------------------------------
// The query's rows in kQBlocks blocks (block b: rows [b n / kQBlocks,
// (b+1) n / kQBlocks)), each with its bounding box.  Every query row is
// coupled to (DTW, Frechet, Euclidean) or has a nearest point in (Hausdorff)
// the candidate, whose points lie in its box, so a block costs at least its
// box's distance to the candidate's box per row; LCSS: a row can only match
// when its block's eps-inflated box meets the candidate's box.
template <int MEAS>
__device__ __forceinline__ float block_bound(const KArgs& a, const float4* qblk, int n, float4 cb,
                                             int m) {
  const int rows_max = MEAS == M_EUCLID ? m : n;  // lock-step: rows 0 .. m-1 only
  float acc = 0.0f;
  int cnt = 0;
  const float e2 = __fmul_ru(a.eps, 1.0f + 1.0f / 1048576.0f);
#pragma unroll
  for (int b = 0; b < kQBlocks; ++b) {
    const int r0 = (int)((long long)b * n / kQBlocks);
    const int r1 = min((int)((long long)(b + 1) * n / kQBlocks), rows_max);
    if (r1 <= r0) continue;
    const float4 bx = qblk[b];
    if (MEAS == M_LCSS) {
      if (cb.z >= __fsub_rd(bx.x, e2) && cb.x <= __fadd_ru(bx.z, e2) &&
          cb.w >= __fsub_rd(bx.y, e2) && cb.y <= __fadd_ru(bx.w, e2))
        cnt += r1 - r0;
      continue;
    }
    const float d = box_box_d2_rd(bx, cb);
    if (MEAS == M_FRECHET || MEAS == M_HAUSDORFF) {
      acc = fmaxf(acc, d);
    } else {
      const float c = (MEAS == M_DTW && a.cost) ? __fsqrt_rd(d) : d;
      acc = __fadd_rd(acc, __fmul_rd((float)(r1 - r0), c));
    }
  }
  return MEAS == M_LCSS ? (float)cnt : acc;
}

// one warp per query: lane b < kQBlocks reduces block b's box
__global__ void qblocks_kernel(const float2* __restrict__ pts, const int64_t* __restrict__ off,
                               int nq, float4* __restrict__ qblk) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq || lane >= kQBlocks) return;
  const int64_t o = off[q];
  const int n = (int)(off[q + 1] - o);
  const int r0 = (int)((long long)lane * n / kQBlocks), r1 = (int)((long long)(lane + 1) * n / kQBlocks);
  float x0 = TSIM_INF, y0 = TSIM_INF, x1 = -TSIM_INF, y1 = -TSIM_INF;
  for (int r = r0; r < r1; ++r) {
    const float2 p = pts[o + r];
    x0 = fminf(x0, p.x);
    y0 = fminf(y0, p.y);
    x1 = fmaxf(x1, p.x);
    y1 = fmaxf(y1, p.y);
  }
  qblk[(size_t)q * kQBlocks + lane] = make_float4(x0, y0, x1, y1);
}

template <int MEAS>
__device__ __forceinline__ float bound1(const KArgs& a, float4 qb, float4 qe, int n, float4 cb,
                                        float4 ce, int m) {
  if (n <= 0 || m <= 0) return MEAS == M_LCSS ? 0.0f : TSIM_INF;  // empty: never a neighbour
  if (MEAS == M_LCSS) {
    // upper bound on the count: 0 when the eps-inflated boxes are disjoint
    const float e2 = __fmul_ru(a.eps, 1.0f + 1.0f / 1048576.0f);
    bool ov = cb.z >= __fsub_rd(qb.x, e2) && cb.x <= __fadd_ru(qb.z, e2) &&
              cb.w >= __fsub_rd(qb.y, e2) && cb.y <= __fadd_ru(qb.w, e2);
    return ov ? (float)min(n, m) : 0.0f;
  }
  if (MEAS == M_HAUSDORFF) {
    // the extreme point of either set along an axis is at least the
    // difference of the two boxes' edges away from every point of the other
    const float e = fmaxf(fmaxf(absdiff_rd(qb.x, cb.x), absdiff_rd(qb.z, cb.z)),
                          fmaxf(absdiff_rd(qb.y, cb.y), absdiff_rd(qb.w, cb.w)));
    return __fmul_rd(e, e);
  }
  const float first = pd2_rd(qe.x, qe.y, ce.x, ce.y);
  const float last = pd2_rd(qe.z, qe.w, ce.z, ce.w);
  const float bb = box_box_d2_rd(qb, cb);
  if (MEAS == M_FRECHET) return fmaxf(fmaxf(first, last), bb);
  if (MEAS == M_EUCLID) {
    // point i of the candidate is paired with point i of the query; the
    // query's full box contains its first-m-point prefix
    if (n < m) return TSIM_INF;
    if (m == 1) return first;
    if (n == m) return __fadd_rd(__fadd_rd(first, last), __fmul_rd((float)(m - 2), bb));
    return __fadd_rd(first, __fmul_rd((float)(m - 1), bb));
  }
  // DTW: the path has >= max(n,m) cells; (0,0) and (n-1,m-1) are on it
  const int L = max(n, m);
  if (L < 2) return a.cost ? __fsqrt_rd(first) : first;
  if (a.cost) {
    float s = __fadd_rd(__fsqrt_rd(first), __fsqrt_rd(last));
    return __fadd_rd(s, __fmul_rd((float)(L - 2), __fsqrt_rd(bb)));
  }
  return __fadd_rd(__fadd_rd(first, last), __fmul_rd((float)(L - 2), bb));
}

// Order in which candidates are tried as seeds (lower first).  Any order
// gives a valid threshold -- the seeds' exact values -- but a good one gives
// a tight threshold.  Distance measures use their O(1) bound; the LCSS bound
// (min(n, m) unless the eps-inflated boxes are disjoint) hardly ranks, so
// LCSS tries the candidates whose end points lie nearest the query's first.
template <int MEAS>
__device__ __forceinline__ float seed_score(float b, const float4& qe, const float4& ce,
                                            bool ends) {
  if (MEAS != M_LCSS) return b;
  if (b <= 0.0f) return TSIM_INF;  // no match possible
  const float d0x = qe.x - ce.x, d0y = qe.y - ce.y, d1x = qe.z - ce.z, d1y = qe.w - ce.w;
  return d0x * d0x + d0y * d0y + (ends ? d1x * d1x + d1y * d1y : 0.0f);
}

// the last points can only be matched to each other when the index window
// lets the ends align (|n - m| <= delta, or no window)
__device__ __forceinline__ bool ends_align(int n, int m, int delta) {
  return delta < 0 || abs(n - m) <= delta;
}

template <int MEAS>
__global__ void __launch_bounds__(kChunk) lb1_kernel(KArgs a) {
  __shared__ unsigned long long keys[kChunk];
  __shared__ SelScratch red;
  __shared__ unsigned long long sel[64];
  const int q = blockIdx.y, chunk = blockIdx.x;
  const int c = chunk * kChunk + threadIdx.x;
  __shared__ float4 qblk[kQBlocks];
  const float4 qb = a.qbox[q], qe = a.qends[q];
  const int n = a.qlen[q];
  if (threadIdx.x < kQBlocks) qblk[threadIdx.x] = a.qblk[(size_t)q * kQBlocks + threadIdx.x];
  __syncthreads();
  unsigned long long key = ~0ull;
  if (c < a.C) {
    const float4 ce = a.cends[c], cb = a.cbox[c];
    const int m = a.clen[c];
    float b = bound1<MEAS>(a, qb, qe, n, cb, ce, m);
    if (n > 0 && m > 0 && (MEAS != M_EUCLID || n >= m)) {
      const float bb = block_bound<MEAS>(a, qblk, n, cb, m);
      b = MEAS == M_LCSS ? fminf(b, fminf(bb, (float)min(n, m))) : fmaxf(b, bb);
    }
    a.lb1[(size_t)q * a.C + c] = b;
    key = pack_key(seed_score<MEAS>(b, qe, ce, ends_align(n, a.clen[c], a.delta)), threadIdx.x);
  }
  keys[threadIdx.x] = key;
  __syncthreads();
  block_select_k(keys, kChunk, a.T, sel, red);
  for (int i = threadIdx.x; i < a.T; i += kChunk) {
    int li = key_index(sel[i]);
    a.chunk_cand[((size_t)q * a.nch + chunk) * a.T + i] = li < 0 ? -1 : chunk * kChunk + li;
  }
}

// ---------------------------------------------------------------------------
// stage B: seeds
// ---------------------------------------------------------------------------
template <int MEAS>
__global__ void __launch_bounds__(kSelThreads) seed_kernel(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SelScratch red;
  __shared__ unsigned long long sel[64];
  const int q = blockIdx.x;
  const int N = a.nch * a.T;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw);
  const int* cc = a.chunk_cand + (size_t)q * N;
  for (int i = threadIdx.x; i < N; i += kSelThreads) {
    int c = cc[i];
    unsigned long long key = ~0ull;
    if (c >= 0) {
      float b = a.lb1[(size_t)q * a.C + c];
      key = pack_key(seed_score<MEAS>(b, a.qends[q], a.cends[c],
                                      ends_align(a.qlen[q], a.clen[c], a.delta)), c);
    }
    keys[i] = key;
  }
  __syncthreads();
  block_select_k(keys, N, a.S, sel, red);
  for (int i = threadIdx.x; i < a.S; i += kSelThreads) {
    int c = key_index(sel[i]);
    a.seeds[(size_t)q * a.S + i] = make_int2(q, c);
    if (c >= 0) atomicOr(a.seedmap + (size_t)q * a.Cw + (c >> 5), 1u << (c & 31));
  }
}

// k-th smallest of the keys a warp holds (SLOTS per lane, ~0 = empty; keys
// unique); ~0 when there are fewer than k
template <int SLOTS>
__device__ unsigned long long warp_kth(unsigned long long (&key)[SLOTS], int k) {
  unsigned long long kth = ~0ull;
  for (int e = 0; e < k; ++e) {
    unsigned long long mn = ~0ull;
    int slot = 0;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s)
      if (key[s] < mn) {
        mn = key[s];
        slot = s;
      }
    const unsigned long long g = warp_min_u64(mn);
    if (g == ~0ull) return ~0ull;
    if (mn == g) {
#pragma unroll
      for (int s = 0; s < SLOTS; ++s)
        if (s == slot) key[s] = ~0ull;
    }
    kth = g;
  }
  return kth;
}

// k-th best seed value -> threshold (DTW/Frechet: widened; LCSS: count).
// One warp per query.
// The seeds' k-th value widened by the FP32 error bound: query q's first
// pruning threshold (a warp, lane = its lane); the query's list counters are
// reset with it.
template <int MEAS>
__device__ void seed_threshold(const KArgs& a, int q, int lane) {
  unsigned long long key[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int i = s * 32 + lane;
    key[s] = ~0ull;
    if (i < a.S && a.seeds[(size_t)q * a.S + i].y >= 0) {
      const float x = a.seed_vals[(size_t)q * a.S + i];
      key[s] = pack_key(MEAS == M_LCSS ? -x : x, i);
    }
  }
  const unsigned long long kth = warp_kth(key, a.k);
  if (lane == 0) {
    float t;
    if (kth == ~0ull) {
      t = MEAS == M_LCSS ? 0.0f : TSIM_INF;  // not enough seeds: keep everything
    } else {
      const float v = ord2f((unsigned)(kth >> 32));
      t = MEAS == M_LCSS ? -v : widen(v, gamma_dp(MEAS, a.qlen[q], a.max_clen));
    }
    if (a.noprune) {
      t = MEAS == M_LCSS ? -TSIM_INF : TSIM_INF;
    } else if (a.thr_in) {  // a threshold shared from an earlier identical query
      const float sv = a.thr_in[q];
      t = MEAS == M_LCSS ? fmaxf(t, sv) : fminf(t, sv);
    }
    a.thr[q] = t;
    a.cnt0[q] = 0;
    a.cnt1[q] = 0;
    a.cnt2[q] = 0;
    a.rcnt[q] = 0;
  }
}

// ---------------------------------------------------------------------------
// stage C: compaction and O(length) bounds
// ---------------------------------------------------------------------------
// The query's sparse table (QTable, bounds.cuh), built in shared or global
// memory by one CTA.
__device__ __forceinline__ void qtable_build(QTable& T, const float2* A, int n, float4* smem) {
  int f_log = 0;
  while ((n + (1 << f_log) - 1) >> f_log > kMaxTable) ++f_log;
  const int nb = (n + (1 << f_log) - 1) >> f_log;
  int levels = 1;
  while ((1 << levels) <= nb) ++levels;
  T.t = smem;
  T.nb = nb;
  T.f_log = f_log;
  T.levels = levels;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    float x0 = TSIM_INF, y0 = TSIM_INF, x1 = -TSIM_INF, y1 = -TSIM_INF;
    const int r0 = b << f_log, r1 = min(n, (b + 1) << f_log);
    for (int r = r0; r < r1; ++r) {
      float2 p = A[r];
      x0 = fminf(x0, p.x);
      y0 = fminf(y0, p.y);
      x1 = fmaxf(x1, p.x);
      y1 = fmaxf(y1, p.y);
    }
    smem[b] = make_float4(x0, y0, x1, y1);
  }
  __syncthreads();
  for (int l = 1; l < levels; ++l) {
    const int h = 1 << (l - 1);
    for (int b = threadIdx.x; b + (1 << l) <= nb; b += blockDim.x) {
      float4 u = smem[(size_t)(l - 1) * nb + b], v = smem[(size_t)(l - 1) * nb + b + h];
      smem[(size_t)l * nb + b] =
          make_float4(fminf(u.x, v.x), fminf(u.y, v.y), fmaxf(u.z, v.z), fmaxf(u.w, v.w));
    }
    __syncthreads();
  }
}

// Bytes of the table buffer of a query of up to max_n rows.
size_t qtable_bytes(int max_n) { return (size_t)qtable_stride(max_n) * sizeof(float4); }

// One CTA per query: its first pruning threshold (warp 0, from the seeds),
// then its sparse table and, for lock-step Euclidean, its prefix sums in
// global memory (read by the segment bounds of every pair of the query).
template <int MEAS>
__global__ void qtable_global_kernel(KArgs a, int sums) {
  __shared__ double2 part[256];
  const int q = blockIdx.x;
  if (threadIdx.x < 32) seed_threshold<MEAS>(a, q, threadIdx.x);
  const int n = a.qlen[q];
  if (n <= 0 || n > a.max_qlen) return;
  const float2* A = a.qpts + a.qoff[q];
  QTable T;
  qtable_build(T, A, n, a.qtab + (size_t)q * a.tstride);
  if (!sums) return;  // prefix sums: lock-step Euclidean only
  // P[j] = sum of (p_i - p_0) over i = 0 .. j-1, j = 0 .. n, in FP64 (each
  // difference of two floats exact), rounded once to float; a chunk per
  // thread.  The FP64 sums are within n 2^-53 sum |p_i - p_0| of exact;
  // qpe[q] keeps twice that, rounded up.
  __shared__ double2 mag[256];
  float2* P = a.qpf + (size_t)q * (a.max_qlen + 1);
  const double x0 = A[0].x, y0 = A[0].y;
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int j0 = min(n, (int)threadIdx.x * per), j1 = min(n, j0 + per);
  double sx = 0.0, sy = 0.0, ax = 0.0, ay = 0.0;
  for (int j = j0; j < j1; ++j) {
    const double dx = (double)A[j].x - x0, dy = (double)A[j].y - y0;
    sx += dx;
    sy += dy;
    ax += fabs(dx);
    ay += fabs(dy);
  }
  part[threadIdx.x] = make_double2(sx, sy);
  mag[threadIdx.x] = make_double2(ax, ay);
  __syncthreads();
  if (threadIdx.x == 0) {
    double rx = 0.0, ry = 0.0, mx = 0.0, my = 0.0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const double2 v = part[i];
      part[i] = make_double2(rx, ry);
      rx += v.x;
      ry += v.y;
      mx += mag[i].x;
      my += mag[i].y;
    }
    P[n] = make_float2((float)rx, (float)ry);
    // n 2^-53 (1 + 2^-40) max(sum |dx|, sum |dy|), doubled, rounded up
    a.qpe[q] = __double2float_ru(2.0 * (double)n * 1.1102230246251565e-16 * (1.0 + 1e-12) *
                                 fmax(mx, my));
  }
  __syncthreads();
  double rx = part[threadIdx.x].x, ry = part[threadIdx.x].y;
  for (int j = j0; j < j1; ++j) {
    P[j] = make_float2((float)rx, (float)ry);
    rx += (double)A[j].x - x0;
    ry += (double)A[j].y - y0;
  }
}

// LCSS with an index window: column j of any candidate can only match query
// rows [j-delta, j+delta], so its O(length) test needs the box of those rows
// -- one box per j, the same for every candidate.  Built once per query
// from its sparse table, inflated by eps with outward rounding (empty
// windows get an empty box).
__global__ void lcss_env_kernel(KArgs a) {
  const int q = blockIdx.x;
  const int n = a.qlen[q];
  float4* E = a.qenv + (size_t)q * a.env_stride;
  const int cnt = min(a.env_stride, n + a.delta + 1);
  if (n <= 0 || n > a.max_qlen) {
    for (int i = threadIdx.x; i < a.env_stride; i += blockDim.x)
      E[i] = make_float4(-TSIM_INF, -TSIM_INF, TSIM_INF, TSIM_INF);  // no bound: everything in
    return;
  }
  const QTable T = qtable_view(a.qtab + (size_t)q * a.tstride, n);
  const float e2 = __fmul_ru(a.eps, 1.0f + 1.0f / 1048576.0f);
  for (int i = threadIdx.x; i < a.env_stride; i += blockDim.x) {
    const int lo = max(0, i - a.delta), hi = min(n - 1, i + a.delta);
    float4 b = make_float4(TSIM_INF, TSIM_INF, -TSIM_INF, -TSIM_INF);  // empty
    if (i < cnt && lo <= hi) {
      const float4 x = qtable_box(T, lo, hi);
      b = make_float4(__fsub_rd(x.x, e2), __fsub_rd(x.y, e2), __fadd_ru(x.z, e2),
                      __fadd_ru(x.w, e2));
    }
    E[i] = b;
  }
}

// Segment bound of one pair: every column of candidate segment s lies in the
// segment's box, and its band admits only the query rows between the band
// rows of the segment's first and last column, so the column costs at least
// the squared distance between the segment box and the box of those rows
// (DTW: summed over the segment's columns; Frechet and Hausdorff: every
// point is matched, so the maximum over segments; LCSS: a column can only
// match when the boxes, eps-inflated, meet).  Columns 0 and m-1 are the
// exact corner cells for DTW.
// columns of candidate segment s: [seg_first(s), seg_first(s + 1))
__device__ __forceinline__ int seg_first(int s, int m) { return (int)(((long long)s * m) / kSegs); }

// Row side of the segment bounds: the query's rows in kRowSegs segments;
// the rows of a segment admit only columns [clo, chi], so each costs at
// least the distance between the segment's box and the nearest candidate
// segment box meeting those columns.
constexpr int kRowSegs = 32;

__device__ __forceinline__ float row_seg_min(const QTable& T, const float4* sb, int m, int r0,
                                             int r1, int clo, int chi, int& sf) {
  const float4 qx = qtable_box(T, r0, r1);
  while (sf < kSegs - 1 && seg_first(sf + 1, m) <= clo) ++sf;
  float mn = TSIM_INF;
  for (int s = sf; s < kSegs && seg_first(s, m) <= chi; ++s) {
    const float4 b = sb[s];
    if (b.x > b.z) continue;  // empty segment (m < kSegs)
    mn = fminf(mn, box_box_d2_rd(qx, b));
  }
  return mn;
}

// A pair's segment bound is evaluated by a group of kSegs lanes (aligned
// within the warp, all active): lane g takes candidate segment g and query
// row segments 4g .. 4g+3, and the parts meet by shuffles inside the group.
// A lane alone ran the 8 + 32 box lookups of a pair one after the other,
// each waiting on the last (latency-bound: 64 us for 8 queries' 6,251 pairs).
// Sums are rounded downward in a tree, a different order from a sequential
// sum but every partial sum still at most the exact one; the group's lanes
// end with the same value (each level adds the same two operands).
constexpr int kSegGroup = kSegs;
constexpr int kRowPerLane = kRowSegs / kSegGroup;
static_assert(kSegGroup == 8 && kRowSegs % kSegGroup == 0, "one candidate segment per lane");

__device__ __forceinline__ unsigned seg_group_mask() {
  return 0xffu << (threadIdx.x & 31 & ~(kSegGroup - 1));
}
__device__ __forceinline__ float group_sum_rd(float v) {
  const unsigned mk = seg_group_mask();
#pragma unroll
  for (int o = kSegGroup / 2; o; o >>= 1) v = __fadd_rd(v, __shfl_xor_sync(mk, v, o, kSegGroup));
  return v;
}
__device__ __forceinline__ float group_max(float v) {
  const unsigned mk = seg_group_mask();
#pragma unroll
  for (int o = kSegGroup / 2; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(mk, v, o, kSegGroup));
  return v;
}
__device__ __forceinline__ int group_isum(int v) {
  const unsigned mk = seg_group_mask();
#pragma unroll
  for (int o = kSegGroup / 2; o; o >>= 1) v += __shfl_xor_sync(mk, v, o, kSegGroup);
  return v;
}
__device__ __forceinline__ bool group_any(bool v) {
  return (__ballot_sync(seg_group_mask(), v) & seg_group_mask()) != 0u;
}

// t: the pair's pruning threshold; once the candidate segments' part exceeds
// it the row segments are not evaluated.  Called by every lane of a group
// with the same pair; g is the lane within the group.
template <int MEAS>
__device__ float seg_bound(const KArgs& a, int q, int c, int n, int m, float lb1, float t, int g,
                           const QTable& Tq, float4 qbq) {
  if (n > a.max_qlen || n < 1 || m < 1) return lb1;
  const float4* sb = a.csegbox + (size_t)c * kSegs;
  // lock-step Euclidean takes the query's table view and box from the
  // caller (read once per thread: 765 -> 712 M instructions per 64-query
  // chunk); the other measures read them per pair, which keeps their kernels
  // at 48 registers (62 with them held across the loop)
  QTable T = Tq;
  float4 qb = qbq;
  if (MEAS != M_EUCLID) {
    qb = a.qbox[q];
    T = qtable_view(a.qtab + (size_t)q * a.tstride, n);
  }
  if (MEAS == M_EUCLID) {
    // lock-step: column j meets row j only, so segment s (L points) costs at
    // least L times its box's squared distance to the box of the same query
    // rows, and at least |sum of the query's points - sum of the candidate's|^2
    // / L per coordinate (Cauchy-Schwarz); the larger of the two per segment
    if (n < m) return TSIM_INF;
    const float2* ss = a.csegsum + (size_t)c * kSegs;
    const float2* P = a.qpf + (size_t)q * (a.max_qlen + 1);
    const float4 qe = a.qends[q];  // the query's first point: P's origin
    float part = 0.0f;
    const int s = g;
    const int b0 = seg_first(s, m), b1 = seg_first(s + 1, m) - 1;
    if (b1 >= b0) {
      const float L = (float)(b1 - b0 + 1);
      const float4 cb = sb[s];
      const float d = box_box_d2_rd(qtable_box(T, b0, b1), cb);
      const float2 sc = ss[s];
      const float2 f1 = P[b1 + 1], f0 = P[b0];
      const float e64 = a.qpe[q];
      // |sum q - sum c| per coordinate, in FP32 from origin-shifted sums:
      // A = f1 - f0 (the query's, less L p_0), B = sc - L p_0 (the
      // candidate's), D = |A - B|.  Each rounding -- f1, f0, A, t = L p_0, B,
      // D, and the candidate sum's (one float rounding of an FP64 sum) -- is
      // at most 2^-24 of its value, so 2^-22 of the magnitudes below covers
      // them twice over; e64 covers the query's FP64 prefix sums and 2^-30 L
      // max|c| the candidate's (at most L^2 2^-53 max|c|, L <= 2^11).
      auto gap = [&](float a1, float a0, float scv, float p0, float c0, float c1) {
        const float A = a1 - a0, t = L * p0, B = scv - t, D = fabsf(A - B);
        float mgn = __fadd_ru(__fadd_ru(fabsf(a1), fabsf(a0)), __fadd_ru(fabsf(t), fabsf(scv)));
        mgn = __fadd_ru(__fmul_ru(__fadd_ru(mgn, D), 1.0f / 4194304.0f), e64);
        mgn = __fadd_ru(mgn, __fmul_ru(__fmul_ru(L, fmaxf(fabsf(c0), fabsf(c1))), 1.0f / 1073741824.0f));
        return fmaxf(0.0f, __fsub_rd(D, mgn));
      };
      const float ax = gap(f1.x, f0.x, sc.x, qe.x, cb.x, cb.z);
      const float ay = gap(f1.y, f0.y, sc.y, qe.y, cb.y, cb.w);
      // / L as * (1/L within 2 ulp, times 1 - 2^-21 rounded down: below
      // 1/L), no division sequence
      const float rl = __fmul_rd(__fdividef(1.0f, L), 0.99999952f);
      const float cs = __fmul_rd(__fadd_rd(__fmul_rd(ax, ax), __fmul_rd(ay, ay)), rl);
      part = fmaxf(__fmul_rd(L, d), cs);
    }
    return fmaxf(group_sum_rd(part), lb1);
  }
  if (MEAS == M_FRECHET || MEAS == M_HAUSDORFF) {
    // every point of either set is matched to some point of the other
    float mx = lb1;
    const float4 b = sb[g];
    if (!(b.x > b.z)) mx = fmaxf(mx, box_box_d2_rd(qb, b));  // else an empty segment
    mx = group_max(mx);
    if (mx > t) return mx;
    const int L = (n + kRowSegs - 1) / kRowSegs;
#pragma unroll
    for (int k = 0; k < kRowPerLane; ++k) {
      const int r0 = (g * kRowPerLane + k) * L;
      int sf = 0;
      if (r0 < n) mx = fmaxf(mx, row_seg_min(T, sb, m, r0, min(n - 1, r0 + L - 1), 0, m - 1, sf));
    }
    return group_max(mx);
  }
  if (MEAS == M_LCSS) {
    const float e2 = __fmul_ru(a.eps, 1.0f + 1.0f / 1048576.0f);
    int count = 0;
    const int s = g;
    const int b0 = (int)((long long)s * m / kSegs), b1 = (int)((long long)(s + 1) * m / kSegs) - 1;
    int lo = 0, hi = n - 1;
    if (a.delta >= 0) {
      lo = max(0, b0 - a.delta);
      hi = min(n - 1, b1 + a.delta);
    }
    if (b1 >= b0 && lo <= hi) {
      const float4 qx = qtable_box(T, lo, hi), b = sb[s];
      if (b.z >= __fsub_rd(qx.x, e2) && b.x <= __fadd_ru(qx.z, e2) && b.w >= __fsub_rd(qx.y, e2) &&
          b.y <= __fadd_ru(qx.w, e2))
        count = b1 - b0 + 1;
    }
    count = group_isum(count);
    return fminf(lb1, (float)min(count, min(n, m)));
  }
  // DTW
  const float4 qe = a.qends[q], ce = a.cends[c];
  if (m == 1) {
    float d = pd2_rd(qe.x, qe.y, ce.x, ce.y);
    float acc = a.cost ? __fsqrt_rd(d) : d;
    if (n > 1) {
      float d2 = pd2_rd(qe.z, qe.w, ce.x, ce.y);
      acc = __fadd_rd(acc, a.cost ? __fsqrt_rd(d2) : d2);
    }
    return fmaxf(acc, lb1);
  }
  float corners;
  {
    float d0 = pd2_rd(qe.x, qe.y, ce.x, ce.y), d1 = pd2_rd(qe.z, qe.w, ce.z, ce.w);
    corners = a.cost ? __fadd_rd(__fsqrt_rd(d0), __fsqrt_rd(d1)) : __fadd_rd(d0, d1);
  }
  const int w = band_w(n, m, a.band_pct);
  const bool banded = w >= 0 && n > 1;
  const long long W = banded ? (long long)w * (min(n, m) - 1) : 0;
  // columns 1 .. m-2 in the candidate's segments, each at least its box's
  // distance to the box of the query rows its band admits
  float part = 0.0f;
  bool infeasible = false;
  {
    const int s = g;
    const int b0 = max(1, (int)((long long)s * m / kSegs));
    const int b1 = min(m - 2, (int)((long long)(s + 1) * m / kSegs) - 1);
    if (b1 >= b0) {
      int lo = 0, hi = n - 1;
      if (banded) {
        lo = max(0, floordiv_i((long long)b0 * (n - 1) - W + (m - 2), m - 1));  // ceil
        hi = min(n - 1, floordiv_i((long long)b1 * (n - 1) + W, m - 1));
      }
      if (lo > hi) {
        infeasible = true;  // a column with no admissible row
      } else {
        const float d = box_box_d2_rd(qtable_box(T, lo, hi), sb[s]);
        part = __fmul_rd((float)(b1 - b0 + 1), a.cost ? __fsqrt_rd(d) : d);
      }
    }
  }
  if (group_any(infeasible)) return TSIM_INF;
  const float acc = __fadd_rd(corners, group_sum_rd(part));
  if (fmaxf(acc, lb1) > t) return fmaxf(acc, lb1);
  // rows 1 .. n-2, each with at least one path cell inside its band columns
  // (the corner cells of rows 0 and n-1 are already counted); a segment of
  // rows r0..r1 admits columns [lo(r0), hi(r0 + L - 1)], from integer ramps
  // started at this lane's first segment
  float accr = corners;
  if (n > 2) {
    const int L = (n - 2 + kRowSegs - 1) / kRowSegs;
    const long long d = n - 1, sl = (long long)L * (m - 1);
    const long long K = floordiv_i(W, (int)d) + 1;
    const int k0 = g * kRowPerLane;
    // lo numerator at row 1 + k0 L, hi numerator at row (k0 + 1) L
    long long xl = (long long)(m - 1) - W + (d - 1) + K * d + (long long)k0 * sl;
    long long xh = (long long)L * (m - 1) + W + (long long)k0 * sl;
    int ql, rl, qh, rh, sq, sr;
    divmod_floor(xl, (int)d, ql, rl);
    divmod_floor(xh, (int)d, qh, rh);
    divmod_floor(sl, (int)d, sq, sr);
    float pr = 0.0f;
    int sf = 0;
    bool none = false;
#pragma unroll
    for (int k = 0; k < kRowPerLane; ++k) {
      const int r0 = 1 + (k0 + k) * L;
      if (r0 > n - 2) break;
      const int r1 = min(n - 2, r0 + L - 1);
      int clo = 0, chi = m - 1;
      if (banded) {
        clo = max(0, ql - (int)K);
        chi = min(m - 1, qh);
        ql += sq;
        rl += sr;
        if (rl >= d) rl -= (int)d, ++ql;
        qh += sq;
        rh += sr;
        if (rh >= d) rh -= (int)d, ++qh;
      }
      if (chi < clo) {  // rows with no admissible column
        none = true;
        break;
      }
      const float mn = row_seg_min(T, sb, m, r0, r1, clo, chi, sf);
      pr = __fadd_rd(pr, __fmul_rd((float)(r1 - r0 + 1), a.cost ? __fsqrt_rd(mn) : mn));
    }
    if (group_any(none)) return TSIM_INF;
    accr = __fadd_rd(corners, group_sum_rd(pr));
  }
  return fmaxf(fmaxf(acc, accr), lb1);
}

// Append the pair to a per-query list, aggregated over a block of kChunk
// threads (every thread of the block calls it): warp counts through shared
// memory, one atomic per block.  A query's list has one counter; with an
// atomic per warp, a 1M-candidate scan queued on it (compact_kernel: 311 us
// for 16 queries x 1M candidates at 12 % SM throughput; 86 us per block).
__device__ __forceinline__ void block_append(bool take, int* count, int* list, int value) {
  __shared__ int wbase[kChunk / 32];
  __shared__ int bbase;
  const unsigned ball = __ballot_sync(0xffffffffu, take);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wbase[warp] = __popc(ball);
  __syncthreads();
  if (threadIdx.x == 0) {
    int total = 0;
#pragma unroll
    for (int w = 0; w < kChunk / 32; ++w) {
      const int n = wbase[w];
      wbase[w] = total;
      total += n;
    }
    bbase = total ? atomicAdd(count, total) : 0;
  }
  __syncthreads();
  if (take) list[bbase + wbase[warp] + __popc(ball & ((1u << lane) - 1))] = value;
}

// Stage A, first half: the pairs the O(1) bound keeps (seeds excluded) are
// listed (in list2, free until the O(length) stage) ...
template <int MEAS>
__global__ void __launch_bounds__(kChunk) compact_kernel(KArgs a) {
  const int q = blockIdx.y;
  const int c = blockIdx.x * kChunk + threadIdx.x;
  const float t = a.thr[q];
  bool pass = false;
  if (c < a.C) {
    const bool seeded = (a.seedmap[(size_t)q * a.Cw + (c >> 5)] >> (c & 31)) & 1u;
    const float b = a.lb1[(size_t)q * a.C + c];
    pass = !seeded && (MEAS == M_LCSS ? (b >= t) : (b <= t));
  }
  block_append(pass, a.cnt0 + q, a.list2 + (size_t)q * a.C, c);
}

// ... and their segment bounds are computed with every lane of a warp busy
// (the O(1) bound keeps few pairs of a chunk).  The bound is kept in place of
// the O(1) bound: the O(length) stage and the round-1 order use the tighter
// of it and their own.
template <int MEAS>
__global__ void __launch_bounds__(256) segfilter_kernel(KArgs a) {
  const int q = blockIdx.y;
  const int cnt = a.cnt0[q];
  const float t = a.thr[q];
  const int n = a.qlen[q];
  const int g = threadIdx.x & (kSegGroup - 1);
  const int per_block = blockDim.x / kSegGroup;  // pairs per block and pass
  // lock-step Euclidean: the query's table view and box once per thread
  QTable T{};
  float4 qb{};
  if (MEAS == M_EUCLID) {
    if (n >= 1 && n <= a.max_qlen) T = qtable_view(a.qtab + (size_t)q * a.tstride, n);
    qb = a.qbox[q];
  }
  const int start = blockIdx.x * per_block;
  const int stride = gridDim.x * per_block;
  for (int e0 = start; e0 < cnt; e0 += stride) {  // uniform per block: whole blocks iterate
    const int e = e0 + (int)threadIdx.x / kSegGroup;
    bool pass = false;
    int c = 0;
    if (e < cnt) {  // uniform per group
      c = a.list2[(size_t)q * a.C + e];
      const float b = a.lb1[(size_t)q * a.C + c];
      const float sbnd = seg_bound<MEAS>(a, q, c, n, a.clen[c], b, t, g, T, qb);
      pass = g == 0 && (MEAS == M_LCSS ? (sbnd >= t) : (sbnd <= t));
      if (pass) a.lb1[(size_t)q * a.C + c] = sbnd;
    }
    block_append(pass, a.cnt1 + q, a.list1 + (size_t)q * a.C, c);
  }
}

// Attempts of a bounded wait on a bulk copy (each may suspend briefly): the
// default, or a smaller count set for tests (0: every wait runs out at once).
constexpr uint32_t kWaitLimitDefault = 1u << 22;
__device__ uint32_t g_wait_limit = kWaitLimitDefault;

template <int MEAS>
__device__ __forceinline__ void lb2_body(const KArgs& a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int q = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cnt = a.cnt1[q];
  if (cnt == 0) return;  // uniform across the CTA
  if (MEAS == M_EUCLID) {
    // no O(length) bound (the exact sum costs the same): the list passes
    // whole, in order, with the segment bounds -- no append per pair (an
    // atomic per pair on the query's counter cost 26 ms per 1,024 x 262,144
    // request)
    // (an empty trajectory on either side leaves a consumed entry, -1)
    const int* L1 = a.list1 + (size_t)q * a.C;
    const bool qok = a.qlen[q] > 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x) {
      const int c = L1[e];
      const bool ok = qok && a.clen[c] > 0;
      a.list2[(size_t)q * a.C + e] = ok ? c : -1;
      a.lb2v[(size_t)q * a.C + e] = ok ? a.lb1[(size_t)q * a.C + c] : TSIM_INF;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.cnt2[q] = cnt;
    return;
  }
  const float2* A = a.qpts + a.qoff[q];
  const int n = a.qlen[q];
  const float4 qb = a.qbox[q];
  const float t = a.thr[q];
  // the query's sparse table of row boxes, built in global memory by
  // qtable_global_kernel (read through L1: a copy in shared memory per CTA
  // held occupancy to 3 CTAs per SM); a query longer than the table was
  // sized for passes every pair (the bound is skipped, never guessed)
  constexpr bool kTable = MEAS == M_DTW || MEAS == M_LCSS;
  const bool use_table = n <= a.max_qlen;
  QTable T;
  if (kTable && use_table) T = qtable_view(a.qtab + (size_t)q * a.tstride, n);
  const float e2 = __fmul_ru(a.eps, 1.0f + 1.0f / 1048576.0f);
  // LCSS: an occupancy grid of the query in shared memory, cells of side
  // gs >= 1.01 eps, each query point marking its cell and the 8 around it.
  // A candidate point within eps (per coordinate) of any query point then
  // lies in a marked cell: its cell index differs from that query point's
  // by at most 1 per axis, the index arithmetic's rounding (< 1e-3 cell)
  // being covered by the 1 % margin.  Points outside the grid match nothing.
  uint32_t* grid = reinterpret_cast<uint32_t*>(smem_raw);
  float gx0 = 0.0f, gy0 = 0.0f, ginv = 0.0f;
  int gnx = 0, gny = 0;
  if (MEAS == M_LCSS && a.eps > 0.0f) {
    float gs = __fmul_ru(a.eps, 1.01f);
    const float W = qb.z - qb.x, H = qb.w - qb.y;
    while ((W / gs + 3.0f) * (H / gs + 3.0f) > 32.0f * kGridWords) gs *= 1.25f;
    gnx = (int)(W / gs) + 3;
    gny = (int)(H / gs) + 3;
    gx0 = qb.x - gs;
    gy0 = qb.y - gs;
    ginv = 1.0f / gs;
    for (int w = threadIdx.x; w < kGridWords; w += blockDim.x) grid[w] = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int cx = min(max((int)((A[i].x - gx0) * ginv), 1), gnx - 2);
      const int cy = min(max((int)((A[i].y - gy0) * ginv), 1), gny - 2);
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int cell = (cy + dy) * gnx + cx + dx;
          atomicOr(grid + (cell >> 5), 1u << (cell & 31));
        }
    }
    __syncthreads();
  }
  // LCSS: the query's window boxes (lcss_env_kernel) in shared memory, next
  // to the grid: a point's test then reads only its own coordinates from
  // global memory
  float4* envs = reinterpret_cast<float4*>(smem_raw + sizeof(uint32_t) * kGridWords);
  if (MEAS == M_LCSS && a.qenv) {
    const float4* Eg = a.qenv + (size_t)q * a.env_stride;
    for (int i = threadIdx.x; i < a.env_stride; i += blockDim.x) envs[i] = Eg[i];
    __syncthreads();
  }
  // DTW: a pair's candidate points come by bulk copy into one of the warp's
  // two shared-memory buffers, the next pair's copy in flight while the
  // current one is bounded (the column loop otherwise waits on each point
  // load).  The copy covers the points rounded out to an even start and
  // count (16-byte alignment); a pair whose range would leave the array, or
  // longer than a buffer, reads global memory as before.  A wait that runs
  // out sets the status word and the pair reads global memory: the bound is
  // the same either way.
  constexpr bool kBulk = MEAS == M_DTW;
  const int cap = kBulk ? a.lb2_cap : 0;
  __shared__ __align__(8) uint64_t bars[kLb2Warps][2];
  float2* bufs = reinterpret_cast<float2*>(smem_raw) + (size_t)warp * 2 * (cap + 2);
  if (kBulk && cap > 0) {
    if (threadIdx.x < 2 * kLb2Warps) mbar_init(&bars[threadIdx.x >> 1][threadIdx.x & 1], 1);
    mbar_init_fence();
    __syncthreads();
  }
  uint32_t phase[2] = {0u, 0u};
  bool pend[2] = {false, false};
  const uint32_t limit = g_wait_limit;
  auto bulk_ok = [&](int64_t o, int m) {
    return cap > 0 && m >= 2 && m <= cap && (o & ~1ll) + (((o & 1) + m + 1) & ~1ll) <= a.ctotal;
  };
  auto drain = [&](int sl) {  // an issued copy not yet waited for
    if (pend[sl]) {
      mbar_wait(&bars[warp][sl], phase[sl], kWaitLimitDefault);
      phase[sl] ^= 1u;
      pend[sl] = false;
    }
  };
  auto issue = [&](int sl, int64_t o, int m) {
    drain(sl);
    const int64_t beg = o & ~1ll;
    const int npts = (int)(((o & 1) + m + 1) & ~1ll);
    if (lane == 0) bulk_load(bufs + sl * (cap + 2), a.cpts + beg, (uint32_t)npts * 8u, &bars[warp][sl]);
    pend[sl] = true;
  };

  // The warp's pairs e, e + S, ...: a pair's candidate index, then its
  // offset, length and segment bound, are dependent loads; they are issued
  // three and two pairs ahead of the pair being bounded, so that the next
  // pair's offset is known when its bulk copy starts and no load latency
  // precedes a column loop.
  const int S = gridDim.x * kLb2Warps;
  const int* L1 = a.list1 + (size_t)q * a.C;
  const float* LB1 = a.lb1 + (size_t)q * a.C;
  int e = blockIdx.x * kLb2Warps + warp;
  int c_cur = e < cnt ? L1[e] : 0;
  int c_nx = e + S < cnt ? L1[e + S] : 0;
  int c_nn = e + 2 * S < cnt ? L1[e + 2 * S] : 0;
  int64_t o_cur = a.coff[c_cur];
  int m_cur = a.clen[c_cur];
  float s_cur = e < cnt ? LB1[c_cur] : 0.0f;
  int64_t o_nx = a.coff[c_nx];
  int m_nx = a.clen[c_nx];
  float s_nx = e + S < cnt ? LB1[c_nx] : 0.0f;
  int slot = 0;
  bool bulk_cur = e < cnt && bulk_ok(o_cur, m_cur);
  if (bulk_cur) issue(0, o_cur, m_cur);
  for (; e < cnt; e += S) {
    const int c = c_cur;
    const int m = m_cur;
    const float sbnd = s_cur;  // the segment bound of stage A
    const int64_t co = o_cur;
    const bool bulk = bulk_cur;
    // the next pair's copy, then the loads two pairs ahead
    const bool bulk_nx = e + S < cnt && bulk_ok(o_nx, m_nx);
    if (bulk_nx) issue(slot ^ 1, o_nx, m_nx);
    const int c_nnn = e + 3 * S < cnt ? L1[e + 3 * S] : 0;
    const int64_t o_nn = a.coff[c_nn];
    const int m_nn = a.clen[c_nn];
    const float s_nn = e + 2 * S < cnt ? LB1[c_nn] : 0.0f;
    const float2* B = a.cpts + co;
    if (bulk) {
      const bool got = __all_sync(0xffffffffu, mbar_wait(&bars[warp][slot], phase[slot], limit));
      if (got) {
        phase[slot] ^= 1u;
        pend[slot] = false;
        B = bufs + slot * (cap + 2) + (co & 1);
      } else if (lane == 0) {
        atomicOr(a.status, 1u);
      }
    }
    c_cur = c_nx;
    o_cur = o_nx;
    m_cur = m_nx;
    s_cur = s_nx;
    bulk_cur = bulk_nx;
    c_nx = c_nn;
    o_nx = o_nn;
    m_nx = m_nn;
    s_nx = s_nn;
    c_nn = c_nnn;
    bool pass;
    float lbv = sbnd;  // the bound (no O(length) bound: stage A's)
    if (n <= 0 || m <= 0) {
      pass = false;
    } else if (MEAS == M_EUCLID) {
      // no O(length) bound: the exact sum costs the same
      pass = true;
    } else if (kTable && !use_table) {
      pass = true;
    } else if (MEAS == M_DTW) {
      // banded LB_Keogh: column j costs at least the distance from c_j to the
      // box of the query rows its band admits; columns 0 and m-1 are the
      // cells (0,0) and (n-1,m-1) every path contains.
      const int w = band_w(n, m, a.band_pct);
      float acc = 0.0f;
      bool feasible = true;
      if (m == 1) {
        if (lane == 0) {
          float d = pd2_rd(A[0].x, A[0].y, B[0].x, B[0].y);
          acc = a.cost ? __fsqrt_rd(d) : d;
          if (n > 1) {
            float d2 = pd2_rd(A[n - 1].x, A[n - 1].y, B[0].x, B[0].y);
            acc = __fadd_rd(acc, a.cost ? __fsqrt_rd(d2) : d2);
          }
        }
      } else {
        if (lane == 0) {
          float d0 = pd2_rd(A[0].x, A[0].y, B[0].x, B[0].y);
          float d1 = pd2_rd(A[n - 1].x, A[n - 1].y, B[m - 1].x, B[m - 1].y);
          acc = a.cost ? __fadd_rd(__fsqrt_rd(d0), __fsqrt_rd(d1)) : __fadd_rd(d0, d1);
        }
        // rows of column j: [ceil((j(n-1)-W)/(m-1)), floor((j(n-1)+W)/(m-1))]
        const bool banded = w >= 0 && n > 1;
        const int D = m - 1;
        const long long W = banded ? (long long)w * (min(n, m) - 1) : 0;
        FloorDiv lo_d, hi_d;
        const int j0 = 1 + lane;
        if (banded) {
          lo_d.init((long long)j0 * (n - 1) - W + D - 1, D);
          hi_d.init((long long)j0 * (n - 1) + W, D);
        }
        const long long inc = 32ll * (n - 1);
        int dq = 0, dr = 0;
        if (banded) divmod_floor(inc, D, dq, dr);
        // no early exit: an infeasible pair's bound is +inf whatever the sum,
        // and a loop without one keeps several point loads in flight.  The
        // band and the cost are compile-time in the loop (a runtime cost test
        // left the rounded square root in every column's code path)
        auto columns = [&](auto band_c, auto eu_c) {
          constexpr bool BAND = decltype(band_c)::value, EU = decltype(eu_c)::value;
#pragma unroll 4
          for (int j = j0; j < m - 1; j += 32) {
            int lo = 0, hi = n - 1;
            if (BAND) {
              lo = max(lo_d.q, 0);
              hi = min(hi_d.q, n - 1);
              lo_d.step(dq, dr);
              hi_d.step(dq, dr);
            }
            if (lo > hi) {  // a column with no admissible row
              feasible = false;
              lo = hi = min(lo, n - 1);
            }
            const float4 bx = qtable_box(T, lo, hi);
            const float2 p = B[j];
            const float d = box_pt_d2_rd(bx.x, bx.y, bx.z, bx.w, p.x, p.y);
            acc = __fadd_rd(acc, EU ? __fsqrt_rd(d) : d);
          }
        };
        using T1 = std::true_type;
        using F0 = std::false_type;
        if (banded) {
          if (a.cost) columns(T1{}, T1{});
          else columns(T1{}, F0{});
        } else {
          if (a.cost) columns(F0{}, T1{});
          else columns(F0{}, F0{});
        }
      }
      for (int o = 16; o; o >>= 1) acc = __fadd_rd(acc, __shfl_xor_sync(0xffffffffu, acc, o));
      feasible = __all_sync(0xffffffffu, feasible);
      lbv = feasible ? fmaxf(acc, sbnd) : TSIM_INF;
      pass = lbv <= t;
    } else if (MEAS == M_FRECHET || MEAS == M_HAUSDORFF) {
      // every point of either trajectory is coupled to (Frechet) or has a
      // nearest point in (Hausdorff) the other, so the squared distance is
      // at least its squared distance to the other's box
      const float4 cb = a.cbox[c];
      float mx = 0.0f;
      for (int j = lane; j < m; j += 32) {
        float2 p = B[j];
        mx = fmaxf(mx, box_pt_d2_rd(qb.x, qb.y, qb.z, qb.w, p.x, p.y));
      }
      for (int i = lane; i < n; i += 32) {
        float2 p = A[i];
        mx = fmaxf(mx, box_pt_d2_rd(cb.x, cb.y, cb.z, cb.w, p.x, p.y));
      }
      for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      lbv = fmaxf(mx, sbnd);
      pass = lbv <= t;
    } else {
      // LCSS: candidate points that can match some query point of their
      // window (rows [j-delta, j+delta]) inside the eps-inflated box
      // (the window's inflated box from the query's row boxes; the whole
      // query's without a window)
      int count = 0;
      const float4* E = a.qenv ? envs : nullptr;
      const float4 qi = make_float4(__fsub_rd(qb.x, e2), __fsub_rd(qb.y, e2), __fadd_ru(qb.z, e2),
                                    __fadd_ru(qb.w, e2));
      const int jend = E ? min(m, a.env_stride) : m;  // columns past n-1+delta match nothing
#pragma unroll 4
      for (int j = lane; j < jend; j += 32) {
        const float4 bx = E ? E[j] : qi;
        const float2 p = B[j];
        if (p.x >= bx.x && p.x <= bx.z && p.y >= bx.y && p.y <= bx.w) {
          const float fx = (p.x - gx0) * ginv, fy = (p.y - gy0) * ginv;
          if (fx >= 0.0f && fy >= 0.0f && fx < (float)gnx && fy < (float)gny) {
            const int cell = (int)fy * gnx + (int)fx;
            if ((grid[cell >> 5] >> (cell & 31)) & 1u) ++count;
          }
        }
      }
      for (int o = 16; o; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
      lbv = fminf((float)min(count, min(n, m)), sbnd);  // an upper bound on the count
      pass = lbv >= t;
    }
    if (pass && lane == 0) {
      int pos = atomicAdd(a.cnt2 + q, 1);
      a.list2[(size_t)q * a.C + pos] = c;
      a.lb2v[(size_t)q * a.C + pos] = lbv;
    }
    __syncwarp();  // every lane is done with this buffer before it is refilled
    slot ^= 1;
  }
  // no copy may be left running into shared memory the next CTA gets
  drain(0);
  drain(1);
}

template <int MEAS>
__global__ void __launch_bounds__(kLb2Warps * 32) lb2_kernel(KArgs a) {
  lb2_body<MEAS>(a);
}

// DTW's at most 48 registers (5 CTAs of 8 warps per SM where shared memory
// allows): the bulk-copy pipeline's state took it to 64 (4 CTAs), and the
// batched workload's step ran 1.4 % slower for it; the few spilled values are
// per-pair state, outside the column loop.  The other measures keep the
// compiler's choice (LCSS spilled in its point loop under the same bound).
__global__ void __launch_bounds__(kLb2Warps * 32, 5) lb2_dtw_kernel(KArgs a) {
  lb2_body<M_DTW>(a);
}

// Round 1: the M best survivors of each query by their O(length) bound
// (most likely to hold the true neighbours) are refined first; their values
// tighten the threshold for the rest.  Taken entries are consumed (-1).
template <int MEAS>
__global__ void __launch_bounds__(kSelThreads) r1_select_kernel(KArgs a) {
  __shared__ SelScratch red;
  __shared__ unsigned long long sel[64];
  const int q = blockIdx.x;
  const int ns = (a.cnt2[q] + kSeg - 1) / kSeg;
  if (threadIdx.x == 0) a.fcnt[q] = 0;  // round 2's list count (refilter_kernel)
  // the segments' M best (seg_select_kernel) hold the query's M best
  block_select_k(a.segkeys + (size_t)q * a.nseg * 64, ns * a.M, a.M, sel, red);
  for (int i = threadIdx.x; i < a.M; i += kSelThreads) {
    const int pos = key_index(sel[i]);
    int c = -1;
    if (pos >= 0) {
      c = a.list2[(size_t)q * a.C + pos];
      a.list2[(size_t)q * a.C + pos] = -1;
    }
    a.r1pairs[(size_t)q * a.M + i] = make_int2(q, c);
  }
}

// k-th best of seeds and round 1 -> tightened threshold (never looser).
// One warp per query.
// k-th best of seeds and round 1 -> tightened threshold (never looser), for
// query q (a warp, lane = its lane)
template <int MEAS>
__device__ float round1_threshold(const KArgs& a, int q, int lane) {
  unsigned long long key[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int i = s * 32 + lane;
    key[s] = ~0ull;
    if (i < a.S) {
      if (a.seeds[(size_t)q * a.S + i].y >= 0) {
        const float x = a.seed_vals[(size_t)q * a.S + i];
        key[s] = pack_key(MEAS == M_LCSS ? -x : x, i);
      }
    } else if (i < a.S + a.M) {
      if (a.r1pairs[(size_t)q * a.M + i - a.S].y >= 0) {
        const float x = a.r1vals[(size_t)q * a.M + i - a.S];
        key[s] = pack_key(MEAS == M_LCSS ? -x : x, i);
      }
    }
  }
  const unsigned long long kth = warp_kth(key, a.k);
  float t = a.thr[q];
  if (kth != ~0ull && !a.noprune) {
    const float v = ord2f((unsigned)(kth >> 32));
    if (MEAS == M_LCSS)
      t = fmaxf(t, -v);
    else
      t = fminf(t, widen(v, gamma_dp(MEAS, a.qlen[q], a.max_clen)));
  }
  return t;
}

// Round 2: the remaining survivors whose bound passes the tightened
// threshold, into list1 (free after stage C).
template <int MEAS>
__global__ void refilter_kernel(KArgs a) {
  const int q = blockIdx.y;
  const int N = a.cnt2[q];
  // every CTA of the query derives the tightened threshold (a warp's
  // selection over at most 128 values); the first stores it for the later
  // stages
  __shared__ float t_sh;
  if (threadIdx.x < 32) {
    const float tq = round1_threshold<MEAS>(a, q, threadIdx.x);
    if (threadIdx.x == 0) {
      t_sh = tq;
      if (blockIdx.x == 0) a.thr2[q] = tq;
    }
  }
  __syncthreads();
  const float t = t_sh;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N; e += gridDim.x * blockDim.x) {
    const int c = a.list2[(size_t)q * a.C + e];
    if (c < 0) continue;
    const float b = a.lb2v[(size_t)q * a.C + e];
    if (MEAS == M_LCSS ? (b >= t) : (b <= t)) {
      const int pos = atomicAdd(a.fcnt + q, 1);
      a.list1[(size_t)q * a.C + pos] = c;
    }
  }
}

// exclusive scan of fcnt -> off2, total -> npairs (one CTA)
__global__ void __launch_bounds__(1024) scan_kernel(KArgs a) {
  __shared__ int part[1024];
  const int per = (a.nq + 1023) / 1024;
  const int b = threadIdx.x * per, e = min(a.nq, b + per);
  int s = 0;
  for (int i = b; i < e; ++i) s += a.fcnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - s;
  for (int i = b; i < e; ++i) {
    a.off2[i] = run;
    run += a.fcnt[i];
  }
  if (threadIdx.x == 1023) {
    a.off2[a.nq] = part[1023];
    *a.npairs = part[1023];
  }
}

__global__ void flatten_kernel(KArgs a) {
  const int q = blockIdx.y;
  const int cnt = a.fcnt[q], base = a.off2[q];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x)
    a.flat[base + e] = make_int2(q, a.list1[(size_t)q * a.C + e]);
}

// Shape-sorted schedule of the survivor pairs: counting sort by ((query +
// candidate length) / 32, longer length / 16), longest first, so that the
// pairs sharing a warp have similar shapes (a warp runs as long as its
// longest pair) and the pairs with the most anti-diagonals -- a warp-per-pair
// kernel's steps -- start first instead of forming the launch's tail (the
// batched workload's survivor round 0.185 -> 0.178 ms against query length
// first).
constexpr int kShapeBits = 7;  // 128 buckets per key part: total length / 32, longer length / 16
constexpr int kNumShapes = 1 << (2 * kShapeBits);

__device__ __forceinline__ int shape_key(int n, int m) {
  return (min((n + m) >> 5, (1 << kShapeBits) - 1) << kShapeBits) |
         min(max(n, m) >> 4, (1 << kShapeBits) - 1);
}

__global__ void shape_hist_kernel(KArgs a) {
  const int np = *a.npairs;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const int2 pr = a.flat[i];
    atomicAdd(a.shape_cnt + (kNumShapes - 1 - shape_key(a.qlen[pr.x], a.clen[pr.y])), 1);
  }
}

// exclusive scan of the shape histogram in place (one CTA of 1024 threads,
// 16 consecutive buckets per thread read as four int4): warp scans by
// shuffles, then a scan of the 32 warp totals
__global__ void __launch_bounds__(1024) shape_scan_kernel(KArgs a) {
  static_assert(kNumShapes == 1024 * 16, "16 buckets per thread");
  __shared__ int wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int4* h = reinterpret_cast<int4*>(a.shape_cnt) + threadIdx.x * 4;
  int4 v[4];
  int s = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[i] = h[i];
    s += v[i].x + v[i].y + v[i].z + v[i].w;
  }
  int inc = s;  // inclusive scan over the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    wsum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int run = inc - s + (warp > 0 ? wsum[warp - 1] : 0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int4 o;
    o.x = run;
    run += v[i].x;
    o.y = run;
    run += v[i].y;
    o.z = run;
    run += v[i].z;
    o.w = run;
    run += v[i].w;
    h[i] = o;
  }
}

__global__ void shape_scatter_kernel(KArgs a) {
  const int np = *a.npairs;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const int2 pr = a.flat[i];
    const int pos = atomicAdd(a.shape_cnt + (kNumShapes - 1 - shape_key(a.qlen[pr.x], a.clen[pr.y])), 1);
    a.order[pos] = i;
  }
}

// ---------------------------------------------------------------------------
// stage E: final selection, FP64 re-score, sort
// ---------------------------------------------------------------------------
// entry i of a query's refined pairs: seeds, then round 1, then round 2
__device__ __forceinline__ void entry(const KArgs& a, int q, int i, int base, int& c, float& v) {
  if (i < a.S) {
    c = a.seeds[(size_t)q * a.S + i].y;
    v = a.seed_vals[(size_t)q * a.S + i];
  } else if (i < a.S + a.M) {
    c = a.r1pairs[(size_t)q * a.M + i - a.S].y;
    v = a.r1vals[(size_t)q * a.M + i - a.S];
  } else {
    c = a.flat[base + i - a.S - a.M].y;
    v = a.flat_vals[base + i - a.S - a.M];
  }
}

// K best keys of one kSeg-entry segment of each query's list, selected in
// shared memory: MODE 0 the O(length) bounds of the survivors (key index =
// position in list2), MODE 1 the refined values (key index = candidate).
// The per-query selections then run over nseg * K keys instead of the list.
template <int MEAS, int MODE>
__global__ void __launch_bounds__(kSelThreads) seg_select_kernel(KArgs a, int K) {
  __shared__ unsigned long long keys[kSeg];
  __shared__ SelScratch red;
  __shared__ unsigned long long sel[64];
  const int q = blockIdx.y, seg = blockIdx.x;
  const int N = MODE == 0 ? a.cnt2[q] : a.S + a.M + a.fcnt[q];
  const int lo = seg * kSeg;
  if (lo >= N) return;
  const int cnt = min(kSeg, N - lo);
  const int base = MODE == 1 ? a.off2[q] : 0;
  for (int t = threadIdx.x; t < cnt; t += kSelThreads) {
    const int i = lo + t;
    unsigned long long key;
    if (MODE == 0) {
      const float b = a.lb2v[(size_t)q * a.C + i];
      key = pack_key(MEAS == M_LCSS ? -b : b, i);
    } else {
      int c;
      float v;
      entry(a, q, i, base, c, v);
      key = c >= 0 ? pack_key(MEAS == M_LCSS ? -v : v, c) : ~0ull;
    }
    keys[t] = key;
  }
  __syncthreads();
  block_select_k(keys, cnt, K, sel, red);
  unsigned long long* out = a.segkeys + (size_t)q * a.nseg * 64 + (size_t)seg * K;
  for (int t = threadIdx.x; t < K; t += kSelThreads) out[t] = sel[t];
}

template <int MEAS>
__global__ void __launch_bounds__(kSelThreads) final_select_kernel(KArgs a) {
  __shared__ SelScratch red;
  __shared__ unsigned long long sel[64];
  const int q = blockIdx.x;
  const int ns = (a.S + a.M + a.fcnt[q] + kSeg - 1) / kSeg;
  block_select_k(a.segkeys + (size_t)q * a.nseg * 64, ns * a.k, a.k, sel, red);
  if (a.thr_out && threadIdx.x == 0) {
    // the query's final threshold: its k-th refined value (widened by the
    // FP32 error bound; LCSS: the k-th count), valid for any later request
    // with the same query, parameters and database (none: +inf / 0)
    const unsigned long long kk = sel[a.k - 1];
    float t = MEAS == M_LCSS ? 0.0f : TSIM_INF;
    if (key_index(kk) >= 0) {
      const float v = ord2f((unsigned)(kk >> 32));
      t = MEAS == M_LCSS ? -v : widen(v, gamma_dp(MEAS, a.qlen[q], a.max_clen));
    }
    a.thr_out[q] = t;
  }
  if (MEAS == M_LCSS) {
    for (int i = threadIdx.x; i < a.k; i += kSelThreads) {
      int c = key_index(sel[i]);
      a.ids[(size_t)q * a.k + i] = c;
      float cntv = c < 0 ? -1.0f : -ord2f((unsigned)(sel[i] >> 32));
      a.dists[(size_t)q * a.k + i] = cntv;
      if (a.dists64) a.dists64[(size_t)q * a.k + i] = cntv;
    }
    return;
  }
  // the k-th best FP32 value fixes the re-score set (collected by
  // rescore_collect_kernel)
  if (threadIdx.x == 0) {
    a.kthkey[q] = sel[a.k - 1];
    a.rraw[q] = 0;
  }
}

// The re-score set: every refined pair within the FP32 error bound of the
// k-th value (or, when that is infinite, the k best keys).  Segments of the
// list in parallel; members are appended in any order (later stages sort).
template <int MEAS>
__global__ void rescore_collect_kernel(KArgs a) {
  const int q = blockIdx.y;
  const int N = a.S + a.M + a.fcnt[q], base = a.off2[q];
  const unsigned long long kth = a.kthkey[q];
  const float tk = kth == ~0ull ? TSIM_INF : ord2f((unsigned)(kth >> 32));
  const bool finite = tk < TSIM_INF;
  const float tr = widen(tk, gamma_dp(MEAS, a.qlen[q], a.max_clen));
  const int hi = min(N, (blockIdx.x + 1) * kSeg);
  for (int i = blockIdx.x * kSeg + threadIdx.x; i < hi; i += blockDim.x) {
    int c;
    float v;
    entry(a, q, i, base, c, v);
    if (c < 0) continue;
    const bool take = finite ? (v <= tr) : (pack_key(v, c) <= kth);
    if (take) {
      const int p = atomicAdd(a.rraw + q, 1);
      if (p < a.RC) {
        a.rpairs[(size_t)q * a.RC + p] = make_int2(q, c);
        a.rdc[(size_t)q * a.RC + p] = v;  // pairwise measures re-use their FP32 values
      }
    }
  }
}

// pad the re-score set to RC entries, count its members (one thread/query)
__global__ void rescore_pad_kernel(KArgs a) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.nq) return;
  const int rc = min(a.rraw[q], a.RC);
  for (int p = rc; p < a.RC; ++p) a.rpairs[(size_t)q * a.RC + p] = make_int2(q, -1);
  a.rcnt[q] = rc;
}

// Bound on |compensated - FP64| relative to the value, for a path of P
// cells.  DTW: each FP32 cost within 4u (u = 2^-24) and the compensated path
// sum within (4P + 32) u^2 of its terms' sum; Frechet: one cost computed
// from exact differences, within (4P + 32) u^2.  Plus (P + 8) 2^-53 for
// FP64's own rounding, with 25% slack.
__device__ __forceinline__ double gamma_c(int meas, int P) {
  const double u = 1.0 / 16777216.0;
  const double u2 = u * u;
  const double e53 = 1.0 / 9007199254740992.0;
  const double cost = meas == M_DTW ? 4.0 * u : 0.0;
  return (cost + (4.0 * P + 32.0) * u2 + (P + 8.0) * e53) * 1.25;
}

// Rank of each re-score entry in (value, candidate) order: a warp per query,
// the entries staged in shared memory, each lane counting the entries before
// its own (ties by entry index, so ranks are distinct).  kRankWarps queries
// per CTA, at most kMaxRC entries each.
constexpr int kRankWarps = 4;
constexpr int kMaxRC = 256;
struct RankSlot {
  double v[kMaxRC];
  int c[kMaxRC];
  unsigned char ord[kMaxRC];  // entry index by rank
};
__device__ __forceinline__ bool before(double dv, int dc, int di, double v, int c, int i) {
  return dv < v || (dv == v && (dc < c || (dc == c && di < i)));
}
__device__ __forceinline__ int rank_of(const RankSlot& S, int n, int i) {
  int r = 0;
  for (int j = 0; j < n; ++j) r += before(S.v[j], S.c[j], j, S.v[i], S.c[i], i) ? 1 : 0;
  return r;
}

// Order the re-score set by compensated value; pairs whose values are within
// the error bound of a neighbour in that order (chains of them) cannot be
// ordered without FP64 and are sent to the FP64 re-score.
template <int MEAS>
__global__ void __launch_bounds__(32 * kRankWarps) cluster_kernel(KArgs a) {
  __shared__ RankSlot slots[kRankWarps];
  const int lane = threadIdx.x & 31;
  RankSlot& S = slots[threadIdx.x >> 5];
  const int q = blockIdx.x * kRankWarps + (threadIdx.x >> 5);
  if (q >= a.nq) return;
  const int n = min(a.rcnt[q], kMaxRC);
  const int2* rp = a.rpairs + (size_t)q * a.RC;
  const double* rv = a.rdc + (size_t)q * a.RC;
  int2* r64p = a.r64pairs + (size_t)q * a.RC;
  // compensated DTW values: gamma_c; FP32 values: twice their bound
  const double g = compensated_rescore(MEAS) ? gamma_c(MEAS, a.qlen[q] + a.max_clen)
                                             : 2.0 * gamma_dp(MEAS, a.qlen[q], a.max_clen);
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  for (int i = lane; i < n; i += 32) {
    S.v[i] = rv[i];
    S.c[i] = rp[i].y;
  }
  for (int i = lane; i < a.RC; i += 32) r64p[i] = make_int2(q, -1);
  __syncwarp();
  for (int i = lane; i < n; i += 32) S.ord[rank_of(S, n, i)] = (unsigned char)i;
  __syncwarp();
  int sent = 0;
  for (int p = lane; p < n; p += 32) {
    const int i = S.ord[p];
    const double v = S.v[i];
    if (!(v < inf)) continue;  // infeasible: exact
    bool amb = a.force64 != 0;
    if (p > 0) {
      const double u = S.v[S.ord[p - 1]];
      if (v - u <= g * (u + v)) amb = true;
    }
    if (p + 1 < n) {
      const double w = S.v[S.ord[p + 1]];
      if (w < inf && w - v <= g * (v + w)) amb = true;
    }
    if (amb) {
      r64p[i] = rp[i];
      ++sent;
    }
  }
  for (int o = 16; o; o >>= 1) sent += __shfl_xor_sync(0xffffffffu, sent, o);
  if (lane == 0 && sent) atomicAdd(a.n64, sent);
}

// final order: FP64 value for cluster members, compensated value otherwise
// (the two agree in order across clusters); ties by candidate index.  The
// first k entries by rank are the result; a warp per query.
template <int MEAS>
__global__ void __launch_bounds__(32 * kRankWarps) final_sort_kernel(KArgs a) {
  __shared__ RankSlot slots[kRankWarps];
  const int lane = threadIdx.x & 31;
  RankSlot& S = slots[threadIdx.x >> 5];
  const int q = blockIdx.x * kRankWarps + (threadIdx.x >> 5);
  if (q >= a.nq) return;
  const int n = min(a.rcnt[q], kMaxRC);
  const int2* rp = a.rpairs + (size_t)q * a.RC;
  const double* rc = a.rdc + (size_t)q * a.RC;
  const double* r64 = a.r64 + (size_t)q * a.RC;
  const int2* r64p = a.r64pairs + (size_t)q * a.RC;
  for (int i = lane; i < n; i += 32) {
    double d = r64p[i].y >= 0 ? r64[i] : rc[i];
    if (is_squared(MEAS)) d = __dsqrt_rn(d);
    S.v[i] = d;
    S.c[i] = rp[i].y;
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    const int r = rank_of(S, n, i);
    if (r < a.k) {
      const size_t o = (size_t)q * a.k + r;
      a.ids[o] = S.c[i];
      a.dists[o] = __double2float_rn(S.v[i]);
      if (a.dists64) a.dists64[o] = S.v[i];
    }
  }
  for (int e = n + lane; e < a.k; e += 32) {
    const size_t o = (size_t)q * a.k + e;
    a.ids[o] = -1;
    a.dists[o] = TSIM_INF;
    if (a.dists64) a.dists64[o] = __longlong_as_double(0x7ff0000000000000ll);
  }
}

__global__ void clear_u32_kernel(unsigned* p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = 0;
}

// Per-request counters, accumulated on the device (no host sync per chunk):
// counters[2..6] += pairs passing the O(1) bound, the O(length) bound,
// refined pairs, re-scored pairs, FP64 re-scored pairs.
__global__ void stats_kernel(KArgs a, unsigned long long* counters, int with_rescore) {
  unsigned long long c1 = 0, c2 = 0, rc = 0;
  for (int q = threadIdx.x; q < a.nq; q += blockDim.x) {
    c1 += a.cnt1[q];
    c2 += a.cnt2[q];
    rc += with_rescore ? a.rcnt[q] : 0;
  }
  for (int o = 16; o; o >>= 1) {
    c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    rc += __shfl_xor_sync(0xffffffffu, rc, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(counters + 2, c1);
    atomicAdd(counters + 3, c2);
    atomicAdd(counters + 5, rc);
  }
  if (threadIdx.x == 0) {
    atomicAdd(counters + 4, (unsigned long long)(*a.npairs) +
                                (a.brute ? 0ull : (unsigned long long)a.nq * (a.S + a.M)));
    if (with_rescore) atomicAdd(counters + 6, (unsigned long long)(*a.n64));
  }
}

// DP of a pair list: the anti-diagonal kernel for the pairs it can take,
// the round-striped kernel (G lanes x R rows) for the rest
// latency: a round of few pairs (seeds, round 1, re-score), whose launch
// lasts as long as its longest pair.  A step of a warp per pair costs R rows
// of instructions on one warp; two warps or a CTA of 8 per pair spread the
// rows for a barrier per step.  Two warps pay off as long as they need at
// most 2 rows per lane; a CTA once a single warp would need 8 or more FP32
// rows per lane, or 4 or more compensated (two-float) ones.
int run_dp(tsim_ctx* ctx, const KArgs& a, int kind, int G, int R, const DpArgs& d,
           bool latency = false) {
  const bool diag_kind = kind == DP_DTW_SQ || kind == DP_DTW_EU || kind == DP_LCSS ||
                         kind == DP_FRECHET_SQ || kind == DP_DTW_SQC || kind == DP_DTW_EUC ||
                         kind == DP_FRECHET_SQC;
  if (!latency && a.lane_gate > 0 && lane_kind(kind)) {
    // many pairs: a lane per pair, with a latency of one pair's cells but a
    // few instructions per cell; the kernel itself passes a round of fewer
    // than lane_gate pairs (a count only the device knows) on whole
    TSIM_TRY(launch_dp_lane(ctx, kind, d, a.lane_ring, a.lanes, a.nlanes, a.lane_gate));
    DpArgs rest = d;
    rest.order = a.lanes;
    rest.npairs_dev = a.nlanes;
    KArgs b = a;
    b.lane_gate = 0;
    return run_dp(ctx, b, kind, G, R, rest, latency);
  }
  if (!diag_kind || a.rdiag == 0) return launch_dp(ctx, kind, G, R, d, a.max_clen);
  const bool twofloat_kind = kind == DP_DTW_SQC || kind == DP_DTW_EUC || kind == DP_FRECHET_SQC;
  if (a.wave && wave_kind(kind) && !twofloat_kind) {
    // lanes along the anti-diagonal, straight-line blocks of 16 steps: the
    // shortest FP32 step of the warp-per-pair forms (a lone 512 x 486 pair
    // 83 us against 104 on two warps per pair; compensated pairs are faster
    // on two warps, 131 against 203 us), and no masked row slots: the
    // latency rounds and the survivor round (after the lane kernel's gate);
    // pairs with more than 64 cells per anti-diagonal go on to the row-group
    // kernels
    TSIM_TRY(launch_dp_wave(ctx, kind, d, d.max_n > 0 ? d.max_n : a.max_qlen, a.max_clen, latency,
                            a.waves, a.nwaves));
    DpArgs rest = d;
    rest.order = a.waves;
    rest.npairs_dev = a.nwaves;
    KArgs b = a;
    b.wave = 0;
    return run_dp(ctx, b, kind, G, R, rest, latency);
  }
  const bool twofloat = kind == DP_DTW_SQC || kind == DP_DTW_EUC || kind == DP_FRECHET_SQC;
  // Latency rounds (few pairs, one wave) pick the kernel by the pair shape
  // (not by the throughput-tuned R): two warps per pair while 64 lanes need
  // at most 2 rows each, longer shapes a CTA per pair.  640 pairs of up to
  // 512 x 512 points, band 10%: compensated 149 us on two warps against 206
  // on one and 358 on a CTA; FP32 112, 128 and 257 us.  FP32 rounds of more
  // pairs than SM sub-partitions (the batched workload's seeds and round 1,
  // with abandoning) ran slower on two warps, so they keep one.
  const bool w2 = latency && a.rdiag_w2 > 0 && a.rdiag_w2 <= 2 &&
                  (twofloat || d.npairs <= 4 * ctx->num_sms);
  if (!w2 && latency && a.rdiag_cta > 0 && a.rdiag_shape >= (twofloat ? 4 : 8)) {
    // the longest pair needs a CTA, but a round's lengths vary (lognormal
    // Frechet queries): the pairs that fit a warp with up to 8 rows per lane
    // run there, each at its fewest rows, the rest on a CTA per pair from
    // one row per lane up -- instead of every pair at the longest pair's R
    TSIM_TRY(launch_dp_diag(ctx, kind, 1, d, a.max_clen, a.lanes, a.nlanes, a.spill2, a.nspill2, 1,
                            twofloat ? 4 : 8));
    DpArgs rest = d;
    rest.order = a.lanes;
    rest.npairs_dev = a.nlanes;
    TSIM_TRY(launch_dp_diag(ctx, kind, 1, rest, a.max_clen, a.spill, a.nspill, a.spill2,
                            a.nspill2, 8));
  } else if (w2 || (latency && twofloat && a.rdiag_shape >= 2 && a.rdiag_w2 > 0)) {
    // two warps per pair: a compensated row per lane and step, for a barrier
    // of two warps
    TSIM_TRY(launch_dp_diag(ctx, kind, a.rdiag_w2, d, a.max_clen, a.spill, a.nspill, a.spill2,
                            a.nspill2, 2));
  } else {
    // latency rounds start at the smallest R the longest pair admits; the
    // survivor round at the tuned R (which may be smaller: its first pass
    // then runs the narrow-band pairs with fewer rows per lane and passes the
    // others on)
    const int r0 = latency ? std::max(a.rdiag, a.rdiag_shape) : a.rdiag;
    TSIM_TRY(launch_dp_diag(ctx, kind, r0, d, a.max_clen, a.spill, a.nspill, a.spill2,
                            a.nspill2));
  }
  DpArgs sp = d;
  sp.order = a.spill;
  sp.npairs_dev = a.nspill;
  return launch_dp(ctx, kind, G, R, sp, a.max_clen);
}

// the FP32 refine of a pair list: wavefront DP or a pairwise kernel
template <int MEAS>
int refine32(tsim_ctx* ctx, const KArgs& a, int dp32, int G, int R, const DpArgs& d,
             bool latency = false) {
  if (is_dp(MEAS)) return run_dp(ctx, a, dp32, G, R, d, latency);
  PwArgs p{d.qpts, d.qoff, d.cpts, d.coff, d.pairs, d.npairs, d.npairs_dev, d.order, d.out,
           nullptr, d.thr, d.cells};
  return launch_pairwise(ctx, MEAS == M_HAUSDORFF ? TSIM_HAUSDORFF : TSIM_EUCLIDEAN, p);
}

// Stage E (shared by the pruned and the brute-force pipelines): k-th value,
// re-score set, compensated / FP64 re-score, final order, counters.
template <int MEAS>
int finish_knn(tsim_ctx* ctx, KArgs& a, int dpc, int dp64) {
  cudaStream_t s = ctx->stream;
  const int nq = a.nq;
  DpArgs d{};
  d.band_pct = MEAS == M_DTW ? a.band_pct : -1;
  d.max_n = a.max_qlen;
  stage_begin(ctx, TSIM_STAGE_SELECT);
  seg_select_kernel<MEAS, 1><<<dim3(a.nseg, nq), kSelThreads, 0, s>>>(a, a.k);
  final_select_kernel<MEAS><<<nq, kSelThreads, 0, s>>>(a);
  launched(ctx, 2);
  if (MEAS != M_LCSS) {
    rescore_collect_kernel<MEAS><<<dim3(a.nseg, nq), kSelThreads, 0, s>>>(a);
    rescore_pad_kernel<<<(nq + 127) / 128, 128, 0, s>>>(a);
    launched(ctx, 2);
  }
  TSIM_CUDA(cudaGetLastError());
  stage_end(ctx);
  if (MEAS != M_LCSS) {
    stage_begin(ctx, TSIM_STAGE_RESCORE);
    DpArgs r{};
    r.qpts = a.qpts;
    r.qoff = a.qoff;
    r.cpts = a.cpts;
    r.coff = a.coff;
    r.pairs = a.rpairs;
    r.npairs = nq * a.RC;
    r.out64 = a.rdc;
    r.band_pct = d.band_pct;
    r.max_n = a.max_qlen;
    r.delta = -1;
    // compensated FP32 re-score of the set, then FP64 only for the pairs it
    // cannot order (near-ties within the compensated error bound)
    if (compensated_rescore(MEAS)) TSIM_TRY(run_dp(ctx, a, dpc, 32, 1, r, true));
    cluster_kernel<MEAS><<<(nq + kRankWarps - 1) / kRankWarps, 32 * kRankWarps, 0, s>>>(a);
    r.pairs = a.r64pairs;
    r.out64 = a.r64;
    if (MEAS == M_FRECHET) {  // exact FP64 values from the FP32 ones: no FP64 DP
      // a CTA of 8 warps per pair, each pair at the fewest rows per lane its
      // length admits (the pairs are few and up to full rows of 2,041
      // points: latency); longer ones on the striped kernel
      r.aux = a.rdc;
      TSIM_TRY(launch_dp_diag(ctx, DP_FRECHET_WIN, 1, r, a.max_clen, a.spill, a.nspill, a.spill2,
                              a.nspill2, 8));
      DpArgs sp = r;
      sp.order = a.spill;
      sp.npairs_dev = a.nspill;
      TSIM_TRY(launch_dp(ctx, DP_FRECHET_WIN, 32, 1, sp, a.max_clen));
    } else if (is_dp(MEAS)) {
      TSIM_TRY(launch_dp(ctx, dp64, 32, 1, r, a.max_clen));
    } else {
      PwArgs p{a.qpts, a.qoff, a.cpts, a.coff, a.r64pairs, nq * a.RC, nullptr, nullptr, nullptr,
               a.r64, nullptr};
      TSIM_TRY(launch_pairwise64(ctx, MEAS == M_HAUSDORFF ? TSIM_HAUSDORFF : TSIM_EUCLIDEAN, p));
    }
    final_sort_kernel<MEAS><<<(nq + kRankWarps - 1) / kRankWarps, 32 * kRankWarps, 0, s>>>(a);
    TSIM_CUDA(cudaGetLastError());
    launched(ctx, 2);
    stage_end(ctx);
  }
  if (ctx->count_funnel) {  // a synchronising request that reports its funnel
    stats_kernel<<<1, 256, 0, s>>>(a, ctx->dcounters, MEAS != M_LCSS ? 1 : 0);
    TSIM_CUDA(cudaGetLastError());
    launched(ctx);
  }
  return TSIM_OK;
}

// Every pair of a small request refined exactly: the bound stages cost more
// (a chain of dependent launches) than they save.  Seeds and round 1 are
// left empty; the flat list holds all pairs, query by query.
__global__ void brute_setup_kernel(KArgs a) {
  const size_t np = (size_t)a.nq * a.C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < np;
       i += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(i / a.C), c = (int)(i % a.C);
    a.flat[i] = make_int2(q, c);
    if (c == 0) {
      a.off2[q] = q * a.C;
      a.fcnt[q] = a.C;
      a.cnt1[q] = a.C;
      a.cnt2[q] = a.C;
      a.rcnt[q] = 0;
      for (int k = 0; k < a.S; ++k) a.seeds[(size_t)q * a.S + k] = make_int2(q, -1);
      for (int k = 0; k < a.M; ++k) a.r1pairs[(size_t)q * a.M + k] = make_int2(q, -1);
    }
    if (i == 0) *a.npairs = (int)np;
  }
}

template <int MEAS>
int run_brute(tsim_ctx* ctx, KArgs& a, int dp32, int dpc, int dp64) {
  cudaStream_t s = ctx->stream;
  const int nq = a.nq;
  const size_t np = (size_t)nq * a.C;
  TSIM_CUDA(cudaMemsetAsync(a.n64, 0, sizeof(int), s));
  stage_begin(ctx, TSIM_STAGE_FILTER);
  brute_setup_kernel<<<(unsigned)std::min<size_t>((np + 255) / 256, 4096), 256, 0, s>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  stage_end(ctx);
  stage_begin(ctx, TSIM_STAGE_DP_SURVIVORS);
  DpArgs d{};
  d.qpts = a.qpts;
  d.qoff = a.qoff;
  d.cpts = a.cpts;
  d.coff = a.coff;
  d.band_pct = MEAS == M_DTW ? a.band_pct : -1;
  d.max_n = a.max_qlen;
  d.delta = a.delta;
  d.eps = a.eps;
  d.cells = ctx->dcounters + 1;
  d.pairs = a.flat;
  d.npairs = (int)np;
  d.out = a.flat_vals;
  int G, R;
  const int wd = MEAS == M_LCSS ? a.delta : band_w(a.max_qlen, a.max_clen, d.band_pct);
  dp_shape(dp32, a.max_qlen, a.max_clen, wd, G, R);
  TSIM_TRY(refine32<MEAS>(ctx, a, dp32, G, R, d));
  stage_end(ctx);
  return finish_knn<MEAS>(ctx, a, dpc, dp64);
}

template <int MEAS>
int run_knn(tsim_ctx* ctx, KArgs& a, int max_qlen, int dp32, int dpc, int dp64, tsim_stats* st) {
  (void)st;
  if (a.brute) return run_brute<MEAS>(ctx, a, dp32, dpc, dp64);
  cudaStream_t s = ctx->stream;
  const int nq = a.nq;
  dim3 g1(a.nch, nq);
  TSIM_CUDA(cudaMemsetAsync(a.n64, 0, sizeof(int), s));
  stage_begin(ctx, TSIM_STAGE_LB1);
  clear_u32_kernel<<<std::min<size_t>(((size_t)nq * a.Cw + 255) / 256, 4096), 256, 0, s>>>(
      a.seedmap, (size_t)nq * a.Cw);
  lb1_kernel<MEAS><<<g1, kChunk, 0, s>>>(a);
  stage_end(ctx);
  launched(ctx, 2);
  stage_begin(ctx, TSIM_STAGE_SEED);
  const size_t seed_smem = sizeof(unsigned long long) * (size_t)a.nch * a.T;
  if (seed_smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(seed_kernel<MEAS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)seed_smem));
  seed_kernel<MEAS><<<nq, kSelThreads, seed_smem, s>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);

  // launch shape of the DP: longest query against the longest candidate
  DpArgs d{};
  d.qpts = a.qpts;
  d.qoff = a.qoff;
  d.cpts = a.cpts;
  d.coff = a.coff;
  d.band_pct = MEAS == M_DTW ? a.band_pct : -1;
  d.max_n = a.max_qlen;
  d.delta = a.delta;
  d.eps = a.eps;
  d.cells = ctx->dcounters;
  int G, R;
  const int wd = MEAS == M_LCSS ? a.delta : band_w(max_qlen, a.max_clen, d.band_pct);
  dp_shape(dp32, max_qlen, a.max_clen, wd, G, R);

  d.pairs = a.seeds;
  d.npairs = nq * a.S;
  d.out = a.seed_vals;
  // few pairs: one pair per warp, one row per lane (the shortest dependency
  // chain per step; throughput is irrelevant at this size)
  const int Gs = 32, Rs = 1;
  if (a.plain) {
    // the plain form: every pair its own kernel launch from the host
    for (int i = 0; i < nq * a.S; ++i) {
      DpArgs one = d;
      one.pairs = a.seeds + i;
      one.npairs = 1;
      one.out = a.seed_vals + i;
      TSIM_TRY(refine32<MEAS>(ctx, a, dp32, Gs, Rs, one));
    }
  } else {
    TSIM_TRY(refine32<MEAS>(ctx, a, dp32, Gs, Rs, d, true));
  }
  stage_end(ctx);

  stage_begin(ctx, TSIM_STAGE_FILTER);
  qtable_global_kernel<MEAS><<<nq, 256, 0, s>>>(a, MEAS == M_EUCLID);  // threshold, segment bounds
  if (MEAS == M_LCSS && a.qenv) {
    lcss_env_kernel<<<nq, 256, 0, s>>>(a);
    launched(ctx);
  }
  compact_kernel<MEAS><<<g1, kChunk, 0, s>>>(a);
  segfilter_kernel<MEAS><<<dim3(std::max(1, std::min(1024, (32 * ctx->num_sms + nq - 1) / nq)), nq),
                           256, 0, s>>>(a);
  launched(ctx);
  launched(ctx, 2);
  if (MEAS == M_DTW) d.qtab = a.qtab;  // the survivor round: remaining columns' bound
  // CTAs per query of the grid-stride filter kernels: about 8 per SM over the
  // whole request, so a single query against a large database fills the GPU
  const int ch = std::max(1, std::min(65535, (8 * ctx->num_sms + nq - 1) / nq));
  // LCSS: the query's grid and window boxes per CTA, and 4x the CTAs per
  // query (its queries' pair counts vary widely; a CTA's set-up is small)
  const size_t lb2_smem =
      MEAS == M_LCSS   ? sizeof(uint32_t) * kGridWords + sizeof(float4) * (size_t)a.env_stride
      : MEAS == M_DTW ? sizeof(float2) * (size_t)kLb2Warps * 2 * (a.lb2_cap + 2)
                       : 0;
  const int ch2 = MEAS == M_LCSS ? std::max(1, std::min(65535, (32 * ctx->num_sms + nq - 1) / nq))
                                 : ch;
  auto lb2 = MEAS == M_DTW ? lb2_dtw_kernel : lb2_kernel<MEAS>;
  if (lb2_smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(lb2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)lb2_smem));
  lb2<<<dim3(ch2, nq), kLb2Warps * 32, lb2_smem, s>>>(a);
  seg_select_kernel<MEAS, 0><<<dim3(a.nseg, nq), kSelThreads, 0, s>>>(a, a.M);
  r1_select_kernel<MEAS><<<nq, kSelThreads, 0, s>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx, 5);
  stage_end(ctx);

  // round 1: the best survivors by bound, abandon against the seed threshold
  stage_begin(ctx, TSIM_STAGE_DP);
  {
    DpArgs r1 = d;
    r1.pairs = a.r1pairs;
    r1.npairs = nq * a.M;
    r1.out = a.r1vals;
    r1.thr = a.thr;
    r1.qtab = nullptr;  // the best pairs by bound rarely abandon: no remaining-columns bound
    if (a.plain) {
      for (int i = 0; i < nq * a.M; ++i) {
        DpArgs one = r1;
        one.pairs = a.r1pairs + i;
        one.npairs = 1;
        one.out = a.r1vals + i;
        TSIM_TRY(refine32<MEAS>(ctx, a, dp32, Gs, Rs, one));
      }
    } else {
      TSIM_TRY(refine32<MEAS>(ctx, a, dp32, Gs, Rs, r1, true));
    }
  }
  stage_end(ctx);

  stage_begin(ctx, TSIM_STAGE_FILTER);
  refilter_kernel<MEAS><<<dim3(ch, nq), 256, 0, s>>>(a);
  scan_kernel<<<1, 1024, 0, s>>>(a);
  flatten_kernel<<<dim3(ch, nq), 256, 0, s>>>(a);
  TSIM_CUDA(cudaMemsetAsync(a.shape_cnt, 0, sizeof(int) * kNumShapes, s));
  const int sb = ctx->num_sms * 4;
  shape_hist_kernel<<<sb, 256, 0, s>>>(a);
  shape_scan_kernel<<<1, 1024, 0, s>>>(a);
  shape_scatter_kernel<<<sb, 256, 0, s>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx, 6);
  stage_end(ctx);

  stage_begin(ctx, TSIM_STAGE_DP_SURVIVORS);
  d.cells = ctx->dcounters + 1;  // counted apart: the survivor round's roofline
  d.pairs = a.flat;
  d.npairs = nq * a.C;
  d.npairs_dev = a.npairs;
  d.out = a.flat_vals;
  d.thr = a.thr2;
  d.order = a.order;
  if (a.plain) {
    int npairs = 0;
    TSIM_CUDA(cudaMemcpyAsync(&npairs, a.npairs, sizeof(int), cudaMemcpyDeviceToHost, s));
    TSIM_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < npairs; ++i) {
      DpArgs one = d;
      one.pairs = a.flat + i;
      one.npairs = 1;
      one.npairs_dev = nullptr;
      one.order = nullptr;
      one.out = a.flat_vals + i;
      TSIM_TRY(refine32<MEAS>(ctx, a, dp32, Gs, Rs, one));
    }
  } else {
    TSIM_TRY(refine32<MEAS>(ctx, a, dp32, G, R, d));
  }
  stage_end(ctx);

  return finish_knn<MEAS>(ctx, a, dpc, dp64);
}

// Band cells of every (query, candidate) pair: sum over rows of the row's
// band width (DTW), window width (LCSS) or m (Frechet).
__global__ void band_cells_kernel(KArgs a, int meas, unsigned long long* out) {
  const int q = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  long long cells = 0;
  if (c < a.C) {
    const int n = a.qlen[q], m = a.clen[c];
    if (meas == M_FRECHET || (meas == M_DTW && a.band_pct < 0) || (meas == M_LCSS && a.delta < 0)) {
      cells = (long long)n * m;
    } else if (meas == M_LCSS) {
      for (int i = 0; i < n; ++i) {
        int lo = max(0, i - a.delta), hi = min(m - 1, i + a.delta);
        if (hi >= lo) cells += hi - lo + 1;
      }
    } else {
      const int w = band_w(n, m, a.band_pct);
      for (int i = 0; i < n; ++i) {
        int lo, hi;
        band_row(i, n, m, w, lo, hi);
        if (hi >= lo) cells += hi - lo + 1;
      }
    }
  }
  for (int o = 16; o; o >>= 1) cells += __shfl_xor_sync(0xffffffffu, cells, o);
  if ((threadIdx.x & 31) == 0 && cells) atomicAdd(out, (unsigned long long)cells);
}

}  // namespace

int band_cells(tsim_ctx* ctx, const tsim_params* p, const float2* qpts, const int64_t* qoff, int nq,
               tsim_db* db, int64_t* cells_out) {
  KArgs a{};
  a.nq = nq;
  a.C = db->count;
  a.clen = db->len;
  a.band_pct = p->band_pct;
  a.delta = p->delta;
  float4* qbox = arena_take<float4>(ctx, nq);
  float4* qends = arena_take<float4>(ctx, nq);
  int* qlen = arena_take<int>(ctx, nq);
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(ctx->dcounters) + 16;
  TSIM_TRY(summarize(ctx, qpts, qoff, nq, qbox, qends, qlen));
  a.qlen = qlen;
  TSIM_CUDA(cudaMemsetAsync(acc, 0, sizeof(unsigned long long), ctx->stream));
  const int meas = p->measure == TSIM_DTW ? M_DTW : (p->measure == TSIM_LCSS ? M_LCSS : M_FRECHET);
  band_cells_kernel<<<dim3((a.C + 255) / 256, nq), 256, 0, ctx->stream>>>(a, meas, acc);
  TSIM_CUDA(cudaGetLastError());
  unsigned long long h = 0;
  TSIM_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
  *cells_out = (int64_t)h;
  return TSIM_OK;
}

namespace {

// Launch parameters of one knn call (everything but the pointers) and the
// scratch it carves from the arena.
size_t knn_plan(const tsim_params* p, int nq, int max_qlen, const tsim_db* db, KArgs& a) {
  const int C = db->count;
  const int k = p->k;
  a.nq = nq;
  a.C = C;
  a.max_clen = db->max_len;
  a.max_qlen = max_qlen;
  a.tstride = qtable_stride(max_qlen);
  a.env_stride = (p->measure == TSIM_LCSS && p->delta >= 0) ? max_qlen + p->delta + 1 : 0;
  a.k = k;
  a.S = std::min(C, std::min(64, std::max(2 * k, 16)));
  a.M = std::min(64, std::max(2 * k, 32));
  a.nch = (C + kChunk - 1) / kChunk;
  a.T = std::min(kChunk, std::max(1, (2 * a.S + a.nch - 1) / a.nch));
  a.T = std::min(a.T, 64);
  a.plain = (p->flags & TSIM_FLAG_PLAIN) ? 1 : 0;
  a.noprune = (p->flags & TSIM_FLAG_NO_PRUNE) ? 1 : 0;
  {
    // small requests skip the bound stages: their dependent launches cost
    // more than computing every pair (cells or point pairs, upper bound)
    const double pairs = (double)nq * C;
    const double work = pairs * (p->measure == TSIM_EUCLIDEAN ? (double)db->max_len
                                                              : (double)max_qlen * db->max_len);
    const bool small = pairs <= 65536.0 && work <= 2.5e8 && !(p->flags & TSIM_FLAG_ALWAYS_PRUNE);
    a.brute = !a.plain && (a.noprune || small) ? 1 : 0;
  }
  {
    // rows per lane-group of the anti-diagonal kernel: the smallest R whose
    // validity condition holds for every pair shape.  2 w(max(n,m)) (min(n,m)-1)
    // / (n+m-2) grows with both lengths, so the longest query against the
    // longest candidate is the worst case (pairs that still fail are spilled
    // to the striped kernel by the kernel itself).
    const int n = max_qlen, m = db->max_len;
    const int wd = p->measure == TSIM_LCSS ? p->delta
                                           : (p->measure == TSIM_DTW ? band_w(n, m, p->band_pct) : -1);
    a.rdiag = 16;  // none fits the worst case: the widest still takes the shorter pairs
    for (int R : {1, 2, 4, 8, 16})
      if (diag_ok(p->measure == TSIM_LCSS, n, m, wd, R)) {
        a.rdiag = R;
        break;
      }
    a.rdiag_cta = 0;
    for (int R : {1, 2, 4, 8})
      if (diag_ok(p->measure == TSIM_LCSS, n, m, wd, R, 256)) {
        a.rdiag_cta = R;
        break;
      }
    a.rdiag_w2 = 0;
    for (int R : {1, 2, 4})
      if (diag_ok(p->measure == TSIM_LCSS, n, m, wd, R, 64)) {
        a.rdiag_w2 = R;
        break;
      }
    a.rdiag_shape = a.rdiag;
    if (a.plain || (p->flags & TSIM_FLAG_NO_PRUNE)) a.rdiag = 0;
    // the lane-per-pair kernel for survivor rounds of many pairs (pruned and
    // brute force): it wins once the round's total work, not its longest
    // pair, sets the time
    const int kind32 = p->measure == TSIM_LCSS ? DP_LCSS
                       : p->measure == TSIM_FRECHET ? DP_FRECHET_SQ
                       : p->cost ? DP_DTW_EU : DP_DTW_SQ;
    a.lane_ring = lane_ring_for(kind32, n, m, p->measure == TSIM_DTW ? p->band_pct : -1, p->delta);
    a.lane_gate = (a.plain || (p->flags & TSIM_FLAG_NO_LANE_DP)) ? 0 : lane_gate_for(kind32, n, m, p->band_pct, p->delta,
                                         db->ctx ? db->ctx->num_sms : 0);
    a.wave = (a.plain || (p->flags & TSIM_FLAG_NO_WAVE_DP)) ? 0 : 1;
  }
  a.cost = p->cost;
  a.band_pct = p->band_pct;
  a.delta = p->delta;
  a.eps = p->epsilon;
  a.Cw = (C + 31) / 32;
  a.RC = std::min(256, std::max(4 * k, 64));
  a.nseg = (a.S + a.M + C + kSeg - 1) / kSeg;
  a.force64 = (p->flags & TSIM_FLAG_FP64_RESCORE) ? 1 : 0;
  const size_t nqC = (size_t)nq * C;
  size_t need = align256(sizeof(float4) * nq) * 2 + align256(sizeof(int) * nq) +
                align256(sizeof(float) * nqC) + align256(sizeof(int) * nq * a.nch * a.T) +
                align256(sizeof(int2) * nq * a.S) + align256(sizeof(unsigned) * nq * a.Cw) +
                align256(sizeof(float) * nq * a.S) + align256(sizeof(float) * nq) +
                5 * align256(sizeof(int) * (nq + 1)) + 2 * align256(sizeof(int) * nqC) +
                align256(sizeof(int) * 4) + align256(sizeof(int2) * nqC) +
                align256(sizeof(float) * nqC) +
                align256(sizeof(unsigned long long) * nq * (size_t)a.nseg * 64) +
                align256(sizeof(unsigned long long) * nq) + align256(sizeof(int) * nq) +
                2 * align256(sizeof(int2) * nq * a.RC) + 2 * align256(sizeof(double) * nq * a.RC) +
                align256(sizeof(int) * nqC) + align256(sizeof(int) * kNumShapes) + 256 +
                align256(sizeof(float) * nqC) + align256(sizeof(int2) * nq * a.M) +
                align256(sizeof(float) * nq * a.M) + 2 * align256(sizeof(float) * (nq + 1)) +
                align256(sizeof(float4) * (size_t)nq * a.tstride) +
                align256(sizeof(float4) * (size_t)nq * a.env_stride) +
                align256(sizeof(float2) * (size_t)nq * (max_qlen + 1)) + align256(sizeof(float) * nq) +
                align256(sizeof(float4) * (size_t)nq * kQBlocks) +
                4 * align256(sizeof(int) * (size_t)nq * std::max(C, a.RC)) + 4 * 256;
  return need;
}

}  // namespace

size_t knn_scratch_bytes(const tsim_params* p, int nq, int max_qlen, const tsim_db* db) {
  KArgs a{};
  return knn_plan(p, nq, max_qlen, db, a);
}

int knn(tsim_ctx* ctx, const tsim_params* p, const float2* qpts, const int64_t* qoff, int nq,
        int max_qlen, tsim_db* db, int* ids, float* dists, double* dists64, tsim_stats* st,
        const float* thr_in, float* thr_out) {
  TSIM_CHECK_ARG(db->count >= 1, "database is empty");
  KArgs a{};
  const size_t need = knn_plan(p, nq, max_qlen, db, a);
  a.thr_in = thr_in;
  a.thr_out = thr_out;
  if (ctx->rdiag_override >= 0 && !a.plain && !a.noprune) a.rdiag = ctx->rdiag_override;
  TSIM_CHECK_ARG((size_t)a.nch * a.T * sizeof(unsigned long long) <= 200 * 1024,
                 "database too large for one request (seed selection)");
  a.qpts = qpts;
  a.qoff = qoff;
  a.cpts = db->pts;
  a.coff = db->off;
  a.cbox = db->box;
  a.cends = db->ends;
  a.clen = db->len;
  a.ids = ids;
  a.dists = dists;
  a.dists64 = dists64;
  TSIM_TRY(arena_reserve(ctx, need));
  const int C = a.C;
  const size_t nqC = (size_t)nq * C;
  float4* qbox = arena_take<float4>(ctx, nq);
  float4* qends = arena_take<float4>(ctx, nq);
  int* qlen = arena_take<int>(ctx, nq);
  a.qbox = qbox;
  a.qends = qends;
  a.qlen = qlen;
  a.lb1 = arena_take<float>(ctx, nqC);
  a.chunk_cand = arena_take<int>(ctx, (size_t)nq * a.nch * a.T);
  a.seeds = arena_take<int2>(ctx, (size_t)nq * a.S);
  a.seedmap = arena_take<unsigned>(ctx, (size_t)nq * a.Cw);
  a.seed_vals = arena_take<float>(ctx, (size_t)nq * a.S);
  a.thr = arena_take<float>(ctx, nq);
  a.cnt0 = arena_take<int>(ctx, nq + 1);
  a.cnt1 = arena_take<int>(ctx, nq + 1);
  a.cnt2 = arena_take<int>(ctx, nq + 1);
  a.off2 = arena_take<int>(ctx, nq + 1);
  a.rcnt = arena_take<int>(ctx, nq + 1);
  a.list1 = arena_take<int>(ctx, nqC);
  a.list2 = arena_take<int>(ctx, nqC);
  a.npairs = arena_take<int>(ctx, 4);
  a.flat = arena_take<int2>(ctx, nqC);
  a.flat_vals = arena_take<float>(ctx, nqC);
  a.segkeys = arena_take<unsigned long long>(ctx, (size_t)nq * a.nseg * 64);
  a.kthkey = arena_take<unsigned long long>(ctx, nq);
  a.rraw = arena_take<int>(ctx, nq);
  a.rpairs = arena_take<int2>(ctx, (size_t)nq * a.RC);
  a.r64 = arena_take<double>(ctx, (size_t)nq * a.RC);
  a.rdc = arena_take<double>(ctx, (size_t)nq * a.RC);
  a.r64pairs = arena_take<int2>(ctx, (size_t)nq * a.RC);
  a.n64 = arena_take<int>(ctx, 4);
  a.lb2v = arena_take<float>(ctx, nqC);
  a.r1pairs = arena_take<int2>(ctx, (size_t)nq * a.M);
  a.r1vals = arena_take<float>(ctx, (size_t)nq * a.M);
  a.thr2 = arena_take<float>(ctx, nq + 1);
  a.fcnt = arena_take<int>(ctx, nq + 1);
  a.qtab = arena_take<float4>(ctx, (size_t)nq * a.tstride);
  a.qenv = a.env_stride ? arena_take<float4>(ctx, (size_t)nq * a.env_stride) : nullptr;
  a.qpf = arena_take<float2>(ctx, (size_t)nq * (max_qlen + 1));
  a.qpe = arena_take<float>(ctx, nq);
  a.qblk = arena_take<float4>(ctx, (size_t)nq * kQBlocks);
  a.spill = arena_take<int>(ctx, (size_t)nq * std::max(C, a.RC));
  a.nspill = arena_take<int>(ctx, 4);
  a.spill2 = arena_take<int>(ctx, (size_t)nq * std::max(C, a.RC));
  a.nspill2 = arena_take<int>(ctx, 4);
  a.lanes = arena_take<int>(ctx, (size_t)nq * std::max(C, a.RC));
  a.nlanes = arena_take<int>(ctx, 4);
  a.waves = arena_take<int>(ctx, (size_t)nq * std::max(C, a.RC));
  a.nwaves = arena_take<int>(ctx, 4);
  a.csegbox = db->segbox;
  a.csegsum = db->segsum;
  // bulk copies of candidate points (DTW's O(length) stage): buffers of up to
  // 512 points, a 16-byte aligned array (the copies' sources are even
  // points), and a database larger than L2, whose points come from HBM: the
  // 1M-trajectory serving database's stage went from 1.84 to 1.35 ms, while
  // the 38 MB batched one's, L2-resident, went from 102 to 113 us (the
  // buffers cut the CTAs per SM from 5 to 3)
  a.ctotal = db->total;
  const bool db_beyond_l2 = (double)db->total * sizeof(float2) > 96.0 * (1 << 20);
  a.lb2_cap = (p->measure == TSIM_DTW && db_beyond_l2 &&
               (reinterpret_cast<uintptr_t>(db->pts) & 15) == 0)
                  ? (std::min(db->max_len, 512) + 1) & ~1
                  : 0;
  a.status = ctx->status;
  a.order = arena_take<int>(ctx, nqC);
  a.shape_cnt = arena_take<int>(ctx, kNumShapes);
  if (!a.shape_cnt) return fail(TSIM_ERR_OUT_OF_MEMORY, "knn scratch carve failed");

  stage_begin(ctx, TSIM_STAGE_SUMMARY);
  TSIM_TRY(summarize(ctx, qpts, qoff, nq, qbox, qends, qlen));
  qblocks_kernel<<<(nq + 3) / 4, 128, 0, ctx->stream>>>(qpts, qoff, nq, a.qblk);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  stage_end(ctx);
  switch (p->measure) {
    case TSIM_DTW:
      return run_knn<M_DTW>(ctx, a, max_qlen, p->cost ? DP_DTW_EU : DP_DTW_SQ,
                            p->cost ? DP_DTW_EUC : DP_DTW_SQC, p->cost ? DP_DTW_EU64 : DP_DTW_SQ64,
                            st);
    case TSIM_LCSS:
      return run_knn<M_LCSS>(ctx, a, max_qlen, DP_LCSS, DP_LCSS, DP_LCSS, st);
    case TSIM_FRECHET:
      a.band_pct = -1;
      return run_knn<M_FRECHET>(ctx, a, max_qlen, DP_FRECHET_SQ, DP_FRECHET_SQC, DP_FRECHET_SQ64,
                                st);
    case TSIM_HAUSDORFF:
      a.band_pct = -1;
      return run_knn<M_HAUSDORFF>(ctx, a, max_qlen, 0, 0, 0, st);
    case TSIM_EUCLIDEAN:
      a.band_pct = -1;
      return run_knn<M_EUCLID>(ctx, a, max_qlen, 0, 0, 0, st);
  }
  return fail(TSIM_ERR_UNSUPPORTED, "measure not supported by this path");
}

}  // namespace tsim

using tsim::knn_request;

namespace {

// the autotuned choices a request of this shape would use (part of its graph key)
uint64_t tuned_tag(tsim_ctx* ctx, const tsim_params* p, int nq, int max_qlen, const tsim_db* db) {
  if (ctx->tuning.empty()) return 0;
  auto it = ctx->tuning.find(tsim::tune_key(p, nq, max_qlen, db));
  if (it == ctx->tuning.end()) return 0;
  return 1 + (uint64_t)(it->second.rdiag + 1) * 64 + (uint64_t)it->second.streams;
}

std::vector<uint64_t> graph_key(tsim_ctx* ctx, const tsim_params* p, const void* qpts,
                                const void* qoff, int nq, int max_qlen, const tsim_db* db,
                                const void* ids, const void* dists, const void* d64) {
  uint32_t eps;
  memcpy(&eps, &p->epsilon, 4);
  return {(uint64_t)p->measure, (uint64_t)p->k, (uint64_t)p->cost, (uint64_t)(uint32_t)p->band_pct,
          eps, (uint64_t)(uint32_t)p->delta, p->flags, (uint64_t)nq, (uint64_t)max_qlen,
          (uint64_t)(uintptr_t)db, (uint64_t)db->count, (uint64_t)(uintptr_t)qpts,
          (uint64_t)(uintptr_t)qoff, (uint64_t)(uintptr_t)ids, (uint64_t)(uintptr_t)dists,
          (uint64_t)(uintptr_t)d64, (uint64_t)ctx->concurrency, tuned_tag(ctx, p, nq, max_qlen, db)};
}

std::vector<uint64_t> arena_gens(tsim_ctx* ctx) {
  std::vector<uint64_t> g{ctx->arena_gen};
  for (tsim_ctx* s : ctx->subs) g.push_back(s->arena_gen);
  return g;
}

}  // namespace

// A request is replayed from a captured CUDA graph when the same shape,
// parameters and buffers come again: the first call runs eagerly (sizing
// every scratch arena), the second is captured -- the fork to child streams
// and the join are captured as graph dependencies -- and later calls launch
// the graph.  Graphs are dropped when an arena is reallocated or a database
// is destroyed.  Stats, profiling, the plain form and TSIM_FLAG_NO_GRAPH
// run eagerly.
namespace tsim {
int set_wait_limit(long long attempts) {
  const uint32_t v = attempts < 0 ? kWaitLimitDefault
                                  : (uint32_t)std::min<long long>(attempts, 0xffffffffll);
  TSIM_CUDA(cudaMemcpyToSymbol(g_wait_limit, &v, sizeof(v)));
  return TSIM_OK;
}

int take_device_status(tsim_ctx* ctx) {
  unsigned v = 0;
  if (!ctx->status) return TSIM_OK;
  TSIM_CUDA(cudaMemcpy(&v, ctx->status, sizeof(v), cudaMemcpyDeviceToHost));
  return status_result(ctx, v);
}

int status_result(tsim_ctx* ctx, unsigned v) {
  if (!v) return TSIM_OK;
  TSIM_CUDA(cudaMemset(ctx->status, 0, sizeof(v)));
  if (v & 1u) return fail(TSIM_ERR_TIMEOUT, "a bounded wait on a bulk copy ran out");
  return TSIM_OK;
}
}  // namespace tsim

extern "C" int tsim_knn(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                        const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int* d_ids,
                        float* d_dists, double* d_dists64, tsim_stats* stats) {
  TSIM_CHECK_ARG(ctx && p && db, "NULL ctx, params or database");
  const bool graphable = !stats && !ctx->profiling &&
                         !(p->flags & (TSIM_FLAG_NO_GRAPH | TSIM_FLAG_PLAIN));
  if (!graphable)
    return knn_request(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64, stats);
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  const auto key = graph_key(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64);
  tsim_ctx::GraphEntry* e = nullptr;
  for (auto& g : ctx->graphs)
    if (g.key == key) e = &g;
  if (e && e->exec && e->gens != arena_gens(ctx)) {  // stale: scratch moved
    cudaGraphExecDestroy(e->exec);
    e->exec = nullptr;
    e->seen = 0;
  }
  if (e && e->exec) {
    TSIM_CUDA(cudaSetDevice(ctx->device));
    TSIM_CUDA(cudaGraphLaunch(e->exec, ctx->stream));
    ctx->launches += e->launches;
    return TSIM_OK;
  }
  if (!e) {
    if (ctx->graphs.size() >= 16) {  // bounded cache: drop the oldest
      if (ctx->graphs.front().exec) cudaGraphExecDestroy(ctx->graphs.front().exec);
      ctx->graphs.erase(ctx->graphs.begin());
    }
    ctx->graphs.push_back(tsim_ctx::GraphEntry{});
    e = &ctx->graphs.back();
    e->key = key;
  }
  if (e->seen++ == 0)  // first sighting: eager, sizes the arenas
    return knn_request(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64, stats);
  // capture
  TSIM_CUDA(cudaSetDevice(ctx->device));
  const int64_t before = ctx->launches;
  for (tsim_ctx* s : ctx->subs) s->launches = 0;
  TSIM_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int st = knn_request(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64, nullptr);
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (st != TSIM_OK || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    e->seen = 0;  // fall back to eager execution of this request
    return knn_request(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64, stats);
  }
  cudaGraphExec_t exec = nullptr;
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    e->seen = 0;
    return knn_request(ctx, p, d_qpts, d_qoff, nq, max_qlen, db, d_ids, d_dists, d_dists64, stats);
  }
  int64_t captured = ctx->launches - before;
  for (tsim_ctx* s : ctx->subs) captured += s->launches;
  ctx->launches = before;
  e->exec = exec;
  e->launches = captured;
  e->gens = arena_gens(ctx);
  TSIM_CUDA(cudaGraphLaunch(exec, ctx->stream));
  ctx->launches += captured;
  return TSIM_OK;
}

namespace tsim {

static int ceil_log2(long long v) {
  int l = 0;
  while ((1ll << l) < v) ++l;
  return l;
}

std::vector<int> tune_key(const tsim_params* p, int nq, int max_qlen, const tsim_db* db) {
  const bool dtw = p->measure == TSIM_DTW, lcss = p->measure == TSIM_LCSS;
  return {p->measure, dtw ? p->cost : 0, dtw ? p->band_pct : -1, lcss ? p->delta : -1, p->k,
          ceil_log2(max_qlen), ceil_log2(db->max_len), ceil_log2(db->count), ceil_log2(nq)};
}

int knn_request(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int* d_ids,
                float* d_dists, double* d_dists64, tsim_stats* stats) {
  TSIM_CHECK_ARG(ctx && p && db, "NULL ctx, params or database");
  TSIM_CHECK_ARG(nq >= 1 && max_qlen >= 1, "nq and max_qlen must be >= 1");
  TSIM_CHECK_ARG(d_qpts && d_qoff && d_ids && d_dists, "NULL device pointer");
  TSIM_CHECK_ARG(p->k >= 1 && p->k <= 64, "k must be in 1..64");
  TSIM_CHECK_ARG(p->measure >= TSIM_DTW && p->measure <= TSIM_EUCLIDEAN, "unknown measure");
  TSIM_CHECK_ARG(p->measure != TSIM_LCSS || p->epsilon >= 0.0f, "LCSS epsilon must be >= 0");
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  if (stats) {
    *stats = tsim_stats{};
    TSIM_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  }
  // Queries in chunks: a chunk's pair count keeps the scratch bounded, and
  // chunks run round-robin on up to ctx->concurrency child streams so the
  // latency-bound stages of different chunks overlap (offsets stay absolute
  // into d_qpts, so a chunk is a slice of d_qoff).
  const int64_t kMaxPairs = int64_t(1) << 24;
  constexpr int kMinChunk = 8;
  int qb = (int)std::max<int64_t>(1, std::min<int64_t>(nq, kMaxPairs / std::max(db->count, 1)));
  int want = ctx->concurrency, rforce = -1;
  if (!ctx->tuning.empty()) {  // autotuned choices for this shape class
    auto it = ctx->tuning.find(tune_key(p, nq, max_qlen, db));
    if (it != ctx->tuning.end()) {
      if (it->second.streams > 0) want = it->second.streams;
      rforce = it->second.rdiag;
    }
  }
  int nstreams = std::min(want, std::max(1, nq / kMinChunk));
  if (p->flags & TSIM_FLAG_PLAIN) nstreams = 1;
  if (nstreams > 1) qb = std::min(qb, (nq + nstreams - 1) / nstreams);
  std::vector<tsim_ctx*> lanes{ctx};
  ctx->rdiag_override = rforce;
  if (nstreams > 1) {
    TSIM_TRY(tsim::ensure_subs(ctx, nstreams));
    TSIM_CUDA(cudaEventRecord(ctx->fork_ev, ctx->stream));
    lanes.assign(ctx->subs.begin(), ctx->subs.begin() + nstreams);
    for (tsim_ctx* s : lanes) {
      s->profiling = ctx->profiling;
      s->rdiag_override = rforce;
      TSIM_CUDA(cudaStreamWaitEvent(s->stream, ctx->fork_ev, 0));
    }
  }
  for (tsim_ctx* c : lanes) c->count_funnel = stats != nullptr;
  if (stats)
    for (tsim_ctx* c : lanes)
      TSIM_CUDA(cudaMemsetAsync(c->dcounters + 2, 0, 5 * sizeof(unsigned long long), c->stream));
  tsim_stats acc{};
  int chunk = 0;
  for (int q0 = 0; q0 < nq; q0 += qb, ++chunk) {
    const int nb = std::min(qb, nq - q0);
    tsim_ctx* run = lanes[chunk % lanes.size()];
    int s = tsim::knn(run, p, reinterpret_cast<const float2*>(d_qpts), d_qoff + q0, nb, max_qlen,
                      db, d_ids + (size_t)q0 * p->k, d_dists + (size_t)q0 * p->k,
                      d_dists64 ? d_dists64 + (size_t)q0 * p->k : nullptr, nullptr);
    if (s != TSIM_OK) return s;
  }
  if (nstreams > 1)
    for (int i = 0; i < nstreams; ++i) {
      TSIM_CUDA(cudaEventRecord(ctx->join_ev[i], ctx->subs[i]->stream));
      TSIM_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join_ev[i], 0));
    }
  if (stats) {
    TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
    TSIM_TRY(tsim::take_device_status(ctx));
    for (tsim_ctx* c : lanes) {
      unsigned long long v[5];
      TSIM_CUDA(cudaMemcpy(v, c->dcounters + 2, sizeof(v), cudaMemcpyDeviceToHost));
      acc.pairs_lb1 += (int64_t)v[0];
      acc.pairs_lb2 += (int64_t)v[1];
      acc.pairs_refined += (int64_t)v[2];
      acc.rescored += (int64_t)v[3];
      acc.rescored_fp64 += (int64_t)v[4];
    }
    *stats = acc;
    TSIM_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    TSIM_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.0f;
    TSIM_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    stats->ms = ms;
    stats->pairs = (int64_t)nq * db->count;
  }
  return TSIM_OK;
}

}  // namespace tsim

extern "C" int tsim_knn_host(tsim_ctx* ctx, const tsim_params* p, const tsim_point* h_qpts,
                             const int64_t* h_qoff, int nq, tsim_db* db, int* h_ids,
                             float* h_dists, tsim_stats* stats) {
  TSIM_CHECK_ARG(ctx && p && db && h_qpts && h_qoff && h_ids && h_dists, "NULL argument");
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  TSIM_CHECK_ARG(nq >= 1 && p->k >= 1 && p->k <= 64, "bad nq or k");
  TSIM_CHECK_ARG(h_qoff[0] == 0, "query offsets must start at 0");
  int max_qlen = 0;
  for (int i = 0; i < nq; ++i) {
    TSIM_CHECK_ARG(h_qoff[i + 1] > h_qoff[i], "queries must be non-empty");
    max_qlen = std::max<int64_t>(max_qlen, h_qoff[i + 1] - h_qoff[i]);
  }
  TSIM_CUDA(cudaSetDevice(ctx->device));
  const size_t npts = (size_t)h_qoff[nq];
  const size_t in_bytes = tsim::align256(sizeof(tsim_point) * npts) + tsim::align256(8 * (nq + 1));
  const size_t out_bytes = tsim::align256(sizeof(int) * nq * p->k) + tsim::align256(sizeof(float) * nq * p->k);
  TSIM_TRY(tsim::pinned_reserve(ctx, in_bytes + out_bytes + 256));
  // device staging lives in a separate allocation (the arena is reset by the knn call)
  if (ctx->hstage_cap < in_bytes + out_bytes) {
    if (ctx->hstage) {
      TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
      TSIM_CUDA(cudaFree(ctx->hstage));
      ctx->hstage = nullptr;
      ctx->hstage_cap = 0;
    }
    const size_t cap = std::max(in_bytes + out_bytes, size_t(1) << 20);
    TSIM_CUDA(tsim::dev_malloc(&ctx->hstage, cap));
    ctx->hstage_cap = cap;
  }
  char* hp = (char*)ctx->pinned;
  char* dp = (char*)ctx->hstage;
  memcpy(hp, h_qpts, sizeof(tsim_point) * npts);
  memcpy(hp + tsim::align256(sizeof(tsim_point) * npts), h_qoff, 8 * (nq + 1));
  TSIM_CUDA(cudaMemcpyAsync(dp, hp, in_bytes, cudaMemcpyHostToDevice, ctx->stream));
  int* d_ids = (int*)(dp + in_bytes);
  float* d_d = (float*)(dp + in_bytes + tsim::align256(sizeof(int) * nq * p->k));
  TSIM_TRY(tsim_knn(ctx, p, (const tsim_point*)dp,
                    (const int64_t*)(dp + tsim::align256(sizeof(tsim_point) * npts)), nq, max_qlen,
                    db, d_ids, d_d, nullptr, stats));
  TSIM_CUDA(cudaMemcpyAsync(hp + in_bytes, dp + in_bytes, out_bytes, cudaMemcpyDeviceToHost,
                            ctx->stream));
  // the status word rides with the results (no extra round trip)
  unsigned* h_status = reinterpret_cast<unsigned*>(hp + in_bytes + out_bytes);
  TSIM_CUDA(cudaMemcpyAsync(h_status, ctx->status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            ctx->stream));
  TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
  TSIM_TRY(tsim::status_result(ctx, *h_status));
  memcpy(h_ids, hp + in_bytes, sizeof(int) * nq * p->k);
  memcpy(h_dists, hp + in_bytes + tsim::align256(sizeof(int) * nq * p->k), sizeof(float) * nq * p->k);
  return TSIM_OK;
}

extern "C" int tsim_band_cells(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                               const int64_t* d_qoff, int nq, tsim_db* db, int64_t* cells) {
  TSIM_CHECK_ARG(ctx && p && db && d_qpts && d_qoff && cells && nq >= 1, "bad arguments");
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  TSIM_CHECK_ARG(p->measure == TSIM_DTW || p->measure == TSIM_LCSS || p->measure == TSIM_FRECHET,
                 "band cells are defined for the DP measures");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  TSIM_TRY(tsim::arena_reserve(ctx, tsim::align256(sizeof(float4) * nq) * 2 +
                                        tsim::align256(sizeof(int) * nq) + 256));
  return tsim::band_cells(ctx, p, (const float2*)d_qpts, d_qoff, nq, db, cells);
}

extern "C" int tsim_dp_pairs(tsim_ctx* ctx, const tsim_params* p, int precision, int kernel,
                             const tsim_point* d_qpts, const int64_t* d_qoff, int max_qlen,
                             const tsim_point* d_cpts, const int64_t* d_coff, int max_clen,
                             const int* d_pairs, int npairs, float* d_out32, double* d_out64) {
  using namespace tsim;
  TSIM_CHECK_ARG(ctx && p && d_qpts && d_qoff && d_cpts && d_coff && d_pairs, "NULL argument");
  TSIM_CHECK_ARG(npairs >= 0 && max_qlen >= 1 && max_clen >= 1, "bad sizes");
  TSIM_CHECK_ARG(precision >= 0 && precision <= 2 && kernel >= 0 && kernel <= 6, "bad mode");
  TSIM_CHECK_ARG(precision == 0 ? d_out32 != nullptr : d_out64 != nullptr, "NULL output");
  int kinds[3];
  if (p->measure == TSIM_DTW) {
    kinds[0] = p->cost ? DP_DTW_EU : DP_DTW_SQ;
    kinds[1] = p->cost ? DP_DTW_EUC : DP_DTW_SQC;
    kinds[2] = p->cost ? DP_DTW_EU64 : DP_DTW_SQ64;
  } else if (p->measure == TSIM_FRECHET) {
    kinds[0] = DP_FRECHET_SQ;
    kinds[1] = DP_FRECHET_SQC;
    kinds[2] = DP_FRECHET_SQ64;
  } else if (p->measure == TSIM_LCSS) {
    TSIM_CHECK_ARG(precision == 0, "LCSS counts are exact: precision must be 0");
    kinds[0] = kinds[1] = kinds[2] = DP_LCSS;
  } else {
    return fail(TSIM_ERR_INVALID_ARG, "tsim_dp_pairs: measure must be DTW, LCSS or Frechet");
  }
  TSIM_CUDA(cudaSetDevice(ctx->device));
  if (npairs == 0) return TSIM_OK;
  const int kind = kinds[precision];
  DpArgs d{};
  d.qpts = reinterpret_cast<const float2*>(d_qpts);
  d.qoff = d_qoff;
  d.cpts = reinterpret_cast<const float2*>(d_cpts);
  d.coff = d_coff;
  d.pairs = reinterpret_cast<const int2*>(d_pairs);
  d.npairs = npairs;
  if (precision == 0)  // one output slot: FP32, or FP64 / compensated
    d.out = d_out32;
  else
    d.out64 = d_out64;
  d.band_pct = p->measure == TSIM_DTW ? p->band_pct : -1;
  d.max_n = max_qlen;
  d.delta = p->delta;
  d.eps = p->epsilon;
  const int wd = p->measure == TSIM_LCSS ? p->delta : band_w(max_qlen, max_clen, d.band_pct);
  int Rd = 0;
  for (int R : {1, 2, 4, 8, 16})
    if (diag_ok(p->measure == TSIM_LCSS, max_qlen, max_clen, wd, R)) {
      Rd = R;
      break;
    }
  int G, R;
  dp_shape(kind, max_qlen, max_clen, wd, G, R);
  const bool diag_kind = precision < 2;
  if (kernel == 1 || (kernel == 0 && (!diag_kind || Rd == 0)) || !diag_kind)
    return launch_dp(ctx, kind, G, R, d, max_clen);
  if (Rd == 0) Rd = 16;  // none fits the longest pair: the widest takes the rest
  const int lanes = kernel == 3 ? 256 : 64;  // a CTA of 8 warps, or 2 warps, per pair
  int Rc = 4;  // the smallest R that fits the longest pair
  for (int R2 : {8, 4, 2, 1})  // R = 8 for a CTA only
    if ((R2 < 8 || kernel == 3) && diag_ok(p->measure == TSIM_LCSS, max_qlen, max_clen, wd, R2, lanes))
      Rc = R2;
  TSIM_TRY(arena_reserve(ctx, 4 * align256(sizeof(int) * (size_t)npairs) + 768 +
                                  align256(sizeof(int) * (size_t)lane_sort_buckets())));
  int* spill = arena_take<int>(ctx, npairs);
  int* nspill = arena_take<int>(ctx, 4);
  int* tmp = arena_take<int>(ctx, npairs);
  int* ntmp = arena_take<int>(ctx, 4);
  int* rest = arena_take<int>(ctx, npairs);
  int* nrest = arena_take<int>(ctx, 4);
  int* sorted = arena_take<int>(ctx, npairs);
  int* buckets = arena_take<int>(ctx, lane_sort_buckets());
  if (kernel == 6 && wave_kind(kind)) {  // band-relative first; wider pairs on the others
    TSIM_TRY(launch_dp_wave(ctx, kind, d, max_qlen, max_clen, npairs <= 4 * ctx->num_sms, rest, nrest));
    d.order = rest;
    d.npairs_dev = nrest;
  } else if (kernel == 5 && lane_kind(kind)) {  // a lane per pair first; wider pairs on a warp
    // neighbouring lanes get pairs of one shape
    TSIM_TRY(lane_sort(ctx, d, sorted, buckets));
    d.order = sorted;
    TSIM_TRY(launch_dp_lane(ctx, kind, d,
                            lane_ring_for(kind, max_qlen, max_clen, d.band_pct, d.delta), rest,
                            nrest));
    d.order = rest;
    d.npairs_dev = nrest;
  }
  if (kernel == 3 || kernel == 4)
    TSIM_TRY(launch_dp_diag(ctx, kind, Rc, d, max_clen, spill, nspill, tmp, ntmp,
                            kernel == 3 ? 8 : 2));
  else
    TSIM_TRY(launch_dp_diag(ctx, kind, Rd, d, max_clen, spill, nspill, tmp, ntmp));
  d.order = spill;
  d.npairs_dev = nspill;
  return launch_dp(ctx, kind, G, R, d, max_clen);
}
