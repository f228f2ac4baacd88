// tsim_internal.cuh -- shared host/device internals of libtsim.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <cmath>
#include <string>
#include <map>
#include <vector>

#include "../../include/tsim.h"

#define TSIM_INF __int_as_float(0x7f800000)

// ---------------------------------------------------------------------------
// error reporting (host)
// ---------------------------------------------------------------------------
namespace tsim {

void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

}  // namespace tsim

#define TSIM_CUDA(call)                                                       \
  do {                                                                        \
    cudaError_t _e = (call);                                                  \
    if (_e != cudaSuccess) return tsim::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define TSIM_CHECK_ARG(cond, msg)                                               \
  do {                                                                          \
    if (!(cond)) return tsim::fail(TSIM_ERR_INVALID_ARG, std::string(__func__) + ": " + (msg)); \
  } while (0)

#define TSIM_TRY(call)            \
  do {                            \
    int _s = (call);              \
    if (_s != TSIM_OK) return _s; \
  } while (0)

// Candidate trajectories carry the bounding boxes and point sums of kSegs
// consecutive column segments: segment s covers columns [s*m/kSegs,
// (s+1)*m/kSegs).  At most 32 (one lane per segment builds them).
constexpr int kSegs = 8;
// slot of the context's device counters that holds its status word: bit 0
// is set by a kernel whose bounded wait on a bulk copy ran out
constexpr int kStatusSlot = 40;

// ---------------------------------------------------------------------------
// context: device, stream and a grow-only scratch arena
// ---------------------------------------------------------------------------
struct tsim_db;
struct tsim_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  int num_sms = 0;
  // scratch arena: one device block, bump-allocated per call, reset per call
  char* arena = nullptr;
  size_t arena_cap = 0;
  size_t arena_used = 0;
  bool arena_external = false;  // arena lent by a server's pool (not freed or grown here)
  // pinned host staging for the host-pointer entry points, and their device
  // staging (apart from the arena, which the device-pointer call resets)
  void* pinned = nullptr;
  size_t pinned_cap = 0;
  void* hstage = nullptr;
  size_t hstage_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // instrumentation: kernels launched, and per-stage CUDA-event timing on
  // the context stream when profiling is on
  int64_t launches = 0;
  bool profiling = false;
  cudaEvent_t stage_ev[2 * 64] = {};
  int stage_id[64] = {};
  int nstage_ev = 0;
  double stage_ms[TSIM_STAGE_COUNT] = {};
  int64_t stage_calls[TSIM_STAGE_COUNT] = {};
  unsigned long long* dcounters = nullptr;  // device: [0] DP cells computed, [kStatusSlot] status
  bool count_funnel = false;  // requests add their pruning funnel to dcounters[2..6]
  unsigned* status = nullptr;  // device status word (its own dcounters slot; a chunk context: its parent's)
  // concurrency: a request's queries are split into chunks that run on these
  // child contexts (own stream and arena), forked from and joined back to
  // `stream` with events, so that latency-bound stages of different chunks
  // overlap on the GPU
  int concurrency = 4;
  std::vector<tsim_ctx*> subs;
  cudaEvent_t fork_ev = nullptr;
  std::vector<cudaEvent_t> join_ev;
  // captured request graphs (tsim_knn replays them for repeated requests)
  struct GraphEntry {
    std::vector<uint64_t> key;
    std::vector<uint64_t> gens;  // arena generations of ctx and child contexts at capture
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
    int seen = 0;
  };
  std::vector<GraphEntry> graphs;
  uint64_t arena_gen = 0;  // bumped whenever the arena is reallocated
  // autotuned launch choices per request shape class (tune_key), and the
  // rows per lane-group forced on the next knn() calls (-1: planner's)
  struct TuneVal {
    int rdiag = -1, streams = 0;
    double ms = 0.0;
  };
  std::map<std::vector<int>, TuneVal> tuning;
  int rdiag_override = -1;
  // databases created on this context; destroying the context releases their
  // device memory and detaches them (a later tsim_db_destroy only frees the
  // handle), so destruction order cannot cause a use-after-free
  std::vector<tsim_db*> dbs;
};

struct tsim_db {
  tsim_ctx* ctx = nullptr;
  int count = 0;
  int64_t total = 0;
  int max_len = 0;
  bool owns = false;
  float2* pts = nullptr;      // device [total]
  int64_t* off = nullptr;     // device [count+1]
  float4* box = nullptr;      // device [count] (x0, y0, x1, y1)
  float4* ends = nullptr;     // device [count] (first.x, first.y, last.x, last.y)
  int* len = nullptr;         // device [count]
  float4* segbox = nullptr;   // device [count * kSegs]: boxes of kSegs equal column segments
  float2* segsum = nullptr;   // device [count * kSegs]: sums of those segments' points
  std::vector<int64_t> h_off; // host copy of offsets (lengths for scheduling)
};

namespace tsim {

// Reserve `bytes` (256-byte aligned) of arena scratch.  The arena only grows
// between calls (arena_reserve); inside a call, allocation never reallocates.
int arena_reserve(tsim_ctx* ctx, size_t bytes);
template <class T>
T* arena_take(tsim_ctx* ctx, size_t count) {
  size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
  if (ctx->arena_used + bytes > ctx->arena_cap) return nullptr;
  T* p = reinterpret_cast<T*>(ctx->arena + ctx->arena_used);
  ctx->arena_used += bytes;
  return p;
}
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int pinned_reserve(tsim_ctx* ctx, size_t bytes);
// Every device and pinned-host allocation of the library goes through these,
// so tsim_debug_fail_allocations can make any of them fail as out of memory.
cudaError_t dev_malloc(void** p, size_t bytes);
cudaError_t host_alloc(void** p, size_t bytes);
// debug: fill every arena reservation with 0xff bytes (NaN floats, -1 ints)
// before a call's kernels run, so scratch read before it is written shows
bool debug_canary();
int ensure_subs(tsim_ctx* ctx, int n);

// stage timing: bracket one stage's launches; no-ops unless profiling is on
void stage_begin(tsim_ctx* ctx, int stage);
void stage_end(tsim_ctx* ctx);
int stage_collect(tsim_ctx* ctx);  // synchronises and accumulates pending stages
inline void launched(tsim_ctx* ctx, int n = 1) { ctx->launches += n; }

// ---------------------------------------------------------------------------
// band geometry (host + device), identical to oracle/oracle.c orc_band_*
// ---------------------------------------------------------------------------
__host__ __device__ inline int band_w(int n, int m, int band_pct) {
  if (band_pct < 0) return -1;
  int L = n > m ? n : m;
  const long long v = (long long)band_pct * L + 99;
  return v <= 2147483647ll ? (int)v / 100 : (int)(v / 100);  // 32-bit when it fits
}

__host__ __device__ inline long long floordiv_ll(long long a, long long b) {
  long long q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
  return q;
}

// Columns of row i inside |i*(m-1) - j*(n-1)| <= w*(min(n,m)-1); hi < lo when
// empty; w < 0 gives the whole row.
__host__ __device__ inline void band_row(int i, int n, int m, int w, int& lo, int& hi) {
  if (w < 0 || n <= 1) {
    lo = 0;
    hi = m - 1;
    return;
  }
  long long mn = (n < m ? n : m) - 1;
  long long W = (long long)w * mn;
  long long c = (long long)i * (m - 1);
  long long l = -floordiv_ll(-(c - W), n - 1);
  long long h = floordiv_ll(c + W, n - 1);
  lo = (int)(l < 0 ? 0 : l);
  hi = (int)(h > m - 1 ? m - 1 : h);
}

// LCSS index window |i-j| <= delta (delta < 0: whole row)
__host__ __device__ inline void window_row(int i, int m, int delta, int& lo, int& hi) {
  if (delta < 0) {
    lo = 0;
    hi = m - 1;
    return;
  }
  lo = i - delta < 0 ? 0 : i - delta;
  hi = i + delta > m - 1 ? m - 1 : i + delta;
}

// order-preserving float -> uint32 (total order for non-NaN floats)
__host__ __device__ inline unsigned f2ord(float f) {
#ifdef __CUDA_ARCH__
  unsigned u = __float_as_uint(f);
#else
  unsigned u;
  memcpy(&u, &f, 4);
#endif
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ord2f(unsigned u) {
  u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

// ---------------------------------------------------------------------------
// launch helpers implemented in the .cu files
// ---------------------------------------------------------------------------
// Arguments of the DP kernels, passed by value: kept at 120 bytes.  A
// version at 136 bytes (two more fields) made the serving workload 20 %
// slower (p50 20 -> 24 ms, same build otherwise, same GPU).  The launch rate
// does not depend on the argument size (488K empty launches/s from 64 to 512
// bytes), so the difference lies in the DP kernels' code generation, which
// near their register caps moves with this struct's definition; hence the
// shared output slot and the table stride derived from max_n.
struct DpArgs {
  const float2* qpts;
  const int64_t* qoff;
  const float2* cpts;
  const int64_t* coff;
  const int2* pairs;  // (query, candidate)
  union {             // per pair; a launch writes one of the two:
    float* out;       //   distance (FP32 domain) or LCSS count (FP32 kinds)
    double* out64;    //   FP64 and compensated kinds
  };
  const int* npairs_dev;  // when set, the pair count is min(*npairs_dev, npairs)
  const float* thr;   // per query abandon threshold, or null
  unsigned long long* cells;  // optional: band cells actually computed (atomic)
  const int* order;   // optional: work item w is pair order[w] (shape-sorted schedule)
  const double* aux;  // optional: a value per pair, passed to the cell policy (else eps)
  const float4* qtab; // optional: queries' sparse tables (qtable_stride(max_n) float4 each):
                      //   DTW abandoning adds the remaining columns' bound
  int npairs;
  int band_pct;       // DTW/Frechet band, <0 none
  int delta;          // LCSS window, <0 none
  float eps;          // LCSS threshold
  int buf_len;        // shared-memory values per segment (>= max candidate length)
  int max_n;          // optional: no query of the pairs is longer (0: unknown)
};
static_assert(sizeof(DpArgs) == 120, "DpArgs is passed by value to every DP launch");

enum DpKind {
  DP_DTW_REF = 0,   // Euclidean cost, no FMA: the reference's dtw.cpp arithmetic
  DP_FRECHET_REF,   // Euclidean distance, no FMA: frechet.cpp arithmetic
  DP_LCSS,          // integer LCSS, strict |d| < eps per coordinate
  DP_DTW_SQ,        // squared cost, FMA (error bounded, FP64 re-score after)
  DP_DTW_EU,        // Euclidean cost, FMA
  DP_FRECHET_SQ,    // squared-domain Frechet, FMA
  DP_DTW_SQ64,      // FP64 re-score kinds: the FP64 oracle's arithmetic
  DP_DTW_EU64,
  DP_FRECHET_SQ64,
  DP_DTW_SQC,       // compensated FP32 (hi, lo) re-score kinds
  DP_DTW_EUC,
  DP_FRECHET_SQC,
  DP_FRECHET_WIN,   // exact FP64 Frechet from the pair's FP32 value (aux): FP64 costs
                    // only inside the window that can hold the FP64 optimum
  DP_NUM_KINDS
};

// shape class of a request for the autotuner's table
std::vector<int> tune_key(const tsim_params* p, int nq, int max_qlen, const tsim_db* db);
// one kNN request on device pointers (chunked, on the context's streams)
int knn_request(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int* d_ids,
                float* d_dists, double* d_dists64, tsim_stats* stats);
// scratch bytes one knn() call carves from the arena
size_t knn_scratch_bytes(const tsim_params* p, int nq, int max_qlen, const tsim_db* db);
// thr_in / thr_out (optional, [nq]): pruning thresholds known beforehand
// (an earlier identical query's), and the final ones for later requests
int knn(tsim_ctx* ctx, const tsim_params* p, const float2* qpts, const int64_t* qoff, int nq,
        int max_qlen, tsim_db* db, int* ids, float* dists, double* dists64, tsim_stats* st,
        const float* thr_in = nullptr, float* thr_out = nullptr);
// reference-semantics batch: scratch size and the call on caller-given scratch
size_t ref_scratch_bytes(int num_t, int m, bool* keys_in_smem);
int ref_batch_core(tsim_ctx* ctx, int measure, const float2* d_t1, const float2* d_t2, int num_t,
                   int n, int m, float eps, float* d_out, char* scratch);

int band_cells(tsim_ctx* ctx, const tsim_params* p, const float2* qpts, const int64_t* qoff, int nq,
               tsim_db* db, int64_t* cells_out);

// warp-per-pair refine kernels of Hausdorff and Euclidean (pairwise_knn.cu)
struct PwArgs {
  const float2* qpts;
  const int64_t* qoff;
  const float2* cpts;
  const int64_t* coff;
  const int2* pairs;
  int npairs;
  const int* npairs_dev;
  const int* order;
  float* out;       // FP32 pass: squared Hausdorff / squared Euclidean, +inf if abandoned
  double* out64;    // FP64 pass
  const float* thr; // per query abandon threshold or null
  unsigned long long* cells = nullptr;  // point pairs compared (FP32 pass), or null
};
int launch_pairwise(tsim_ctx* ctx, int measure, const PwArgs& a);
int launch_pairwise64(tsim_ctx* ctx, int measure, const PwArgs& a);

// G lanes per pair (4, 8, 16 or 32), R rows per lane (1, 2, 4 or 8).
int launch_dp(tsim_ctx* ctx, int kind, int G, int R, const DpArgs& a, int max_m);
// Anti-diagonal kernel (dp_diag.cu) for DTW/LCSS/Frechet FP32 and compensated
// kinds: passes with R, 2R, .. rows per lane-group, each taking the pairs the
// previous one could not; pairs no pass takes are left in spill[] (count in
// *nspill) for launch_dp.  tmp/ntmp: a second list of the same size.  max_m
// bounds the candidate length (shared-memory staging).  warps: 1 = a warp
// per pair (R up to 16), > 1 = a CTA of 8 warps per pair (R up to 4; for few,
// long, full-row pairs, where the latency of one pair is the launch's).
// rmax > 0 caps the chain's R (pairs needing more rows go to spill).
int launch_dp_diag(tsim_ctx* ctx, int kind, int R, const DpArgs& a, int max_m, int* spill,
                   int* nspill, int* tmp, int* ntmp, int warps = 1, int rmax = 0);
// Band-relative anti-diagonal kernel (dp_wave.cu) for DTW and Frechet, FP32
// and compensated (wave_kind): a warp per pair, lane p holding the p-th live
// cells of the anti-diagonal, R = 1 or 2 cells per lane as the pair needs; pairs
// whose band holds more than 64 cells per anti-diagonal (or longer than
// 2048 points, or than max_n x max_m) are left in spill[] (count in *nspill).
bool wave_kind(int kind);
// After a synchronisation: TSIM_ERR_TIMEOUT (and the status word cleared) if
// a kernel of ctx or of its chunk contexts (which share its word) set the
// timeout bit, else OK.
int take_device_status(tsim_ctx* ctx);
// The same for a status word value already read on the host.
int status_result(tsim_ctx* ctx, unsigned v);
// Attempts of the bounded waits on bulk copies (< 0: the default); for tests.
int set_wait_limit(long long attempts);
int launch_dp_wave(tsim_ctx* ctx, int kind, const DpArgs& a, int max_n, int max_m, bool latency,
                   int* spill, int* nspill);
// Lane-per-pair kernel (dp_lane.cu) for the FP32 DTW, Frechet and LCSS
// kinds (lane_kind): a lane runs a whole pair in passes of 8 rows, the row
// above a pass in a shared-memory ring of `ring` (64 or 128) values per lane
// (lane_ring_for picks it from the longest pair); pairs wider than the ring,
// or with fewer than two points on a side, are left in spill[] (count in
// *nspill, cleared here).  When the list holds fewer than `gate` pairs (read
// on the device) the kernel computes nothing and copies the whole list, in
// order, to spill[] for the warp-per-pair kernels.
bool lane_kind(int kind);
// order[] := the indices 0 .. a.npairs-1 of a.pairs sorted by shape (longer
// length / 16, shorter length / 16, longest first); counts: lane_sort_buckets() ints
int lane_sort(tsim_ctx* ctx, const DpArgs& a, int* order, int* counts);
int lane_sort_buckets();
// pair count from which a survivor round of pairs up to max_n x max_m runs
// on a lane per pair (band_pct / delta < 0: none)
int lane_gate_for(int kind, int max_n, int max_m, int band_pct, int delta, int num_sms);
int lane_ring_for(int kind, int max_n, int max_m, int band_pct, int delta);
int launch_dp_lane(tsim_ctx* ctx, int kind, const DpArgs& a, int ring, int* spill, int* nspill,
                   int gate = 0);
// the anti-diagonal kernel's validity condition for a pair shape, R rows
// per lane-group and `lanes` lanes per pair
bool diag_ok(bool lcss, int n, int m, int wd, int R, int lanes = 32);

// choose (G, R) for pairs of shape n x m under band w
void dp_shape(int kind, int n, int m, int band_w_or_delta, int& G, int& R);

}  // namespace tsim
