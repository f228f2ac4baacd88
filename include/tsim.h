/*
 * tsim.h -- C ABI of the GB300 trajectory-similarity kNN engine (libtsim.so).
 *
 * Plain C: pointers, sizes and status codes; no C++ or torch types.  Every
 * entry point returns a tsim_status; tsim_last_error() gives the message of
 * the last failure on the calling thread.  Nothing here ever calls exit():
 * the reference's CHECK macro (CudaRuntime1/common.cuh:14-22) terminates the
 * process, this ABI reports instead.
 *
 * Points are `tsim_point {float x, y;}`, the same 8-byte layout as the
 * reference's `struct Point` (CudaRuntime1/common.cuh:9-11).  Trajectory sets
 * are CSR: points[off[t] .. off[t+1]) is trajectory t.
 *
 * Two families of entry points:
 *  - reference-semantics batch calls (tsim_ref_*), one value per query,
 *    reproducing the reference's filter -> top-10 -> refine -> reduce
 *    results bit for bit (DTW, LCSS, Frechet) or from given candidates
 *    (Hausdorff, Euclidean); the reference-named C++ functions in
 *    include/compat/ are thin wrappers over these;
 *  - exact kNN (tsim_knn*): rectangular query x database, variable lengths,
 *    top-k ids and distances, lower-bound pruning that never drops a true
 *    neighbour, a compensated (double-float) FP32 re-score of the survivors
 *    with FP64 for pairs it cannot order; ids ranked by (FP64 distance,
 *    candidate index), LCSS by (count descending, index).
 */
#ifndef TSIM_H
#define TSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TSIM_API __attribute__((visibility("default")))
#else
#define TSIM_API
#endif

typedef struct tsim_point {
  float x, y;
} tsim_point;

typedef enum tsim_status {
  TSIM_OK = 0,
  TSIM_ERR_INVALID_ARG = 1,
  TSIM_ERR_CUDA = 2,
  TSIM_ERR_OUT_OF_MEMORY = 3,
  TSIM_ERR_TIMEOUT = 4, /* a bounded device-side wait ran out */
  TSIM_ERR_UNSUPPORTED = 5,
  TSIM_ERR_BUDGET = 6, /* request exceeds the admission budget */
  TSIM_PENDING = 7,    /* a served request has not finished yet */
  TSIM_ERR_BUSY = 8    /* the server's admission queue is full */
} tsim_status;

typedef enum tsim_measure {
  TSIM_DTW = 0,
  TSIM_LCSS = 1,
  TSIM_FRECHET = 2,
  TSIM_HAUSDORFF = 3,
  TSIM_EUCLIDEAN = 4
} tsim_measure;

typedef enum tsim_cost {
  TSIM_COST_SQEUCLID = 0, /* DTW cell cost |a-b|^2 */
  TSIM_COST_EUCLID = 1    /* DTW cell cost |a-b| (the reference's, dtw.cpp:90) */
} tsim_cost;

/* tsim_params.flags */
#define TSIM_FLAG_NO_PRUNE 0x1u /* compute every pair (no lower bounds) */
#define TSIM_FLAG_PLAIN 0x2u    /* "plain" form: one DP pair per kernel launch */
#define TSIM_FLAG_NO_GRAPH 0x4u /* do not replay through a captured CUDA graph */
#define TSIM_FLAG_FP64_RESCORE 0x8u /* re-score every top-k pair in FP64: distances
                                       bit-identical to an FP64 evaluation */
#define TSIM_FLAG_ALWAYS_PRUNE 0x10u /* run the bound stages even for requests small
                                        enough to refine every pair (the default) */
#define TSIM_FLAG_NO_LANE_DP 0x20u  /* survivor rounds stay on the warp-per-pair DP
                                       kernels even when they hold many pairs (the
                                       lane-per-pair kernel is off); same values */
#define TSIM_FLAG_NO_WAVE_DP 0x40u  /* DTW / Frechet rounds skip the band-relative DP
                                       kernel (lanes along the anti-diagonal) and start
                                       on the row-group ones; same values */
#define TSIM_FLAG_SHARE_THRESHOLDS 0x80u /* server requests: a query's pruning threshold
                                             starts from the final one of an earlier
                                             identical query (same parameters, points and
                                             database), so repeated queries prune at once;
                                             same answers */

typedef struct tsim_params {
  int measure;    /* tsim_measure */
  int k;          /* neighbours per query, 1..64 */
  int cost;       /* DTW only: tsim_cost */
  int band_pct;   /* DTW only: Sakoe-Chiba band, percent of max(n,m); <0 = none */
  float epsilon;  /* LCSS only: per-coordinate match threshold, |dx| < eps */
  int delta;      /* LCSS only: index window |i-j| <= delta; <0 = none */
  unsigned flags; /* TSIM_FLAG_* */
} tsim_params;

typedef struct tsim_stats {
  double ms;              /* device time of the call (CUDA events) */
  int64_t pairs;          /* query x candidate pairs in the request */
  int64_t pairs_lb1;      /* pairs passing the O(1) bound */
  int64_t pairs_lb2;      /* pairs passing the O(length) bound */
  int64_t pairs_refined;  /* pairs that reached the exact DP / distance */
  int64_t cells;          /* DP cells (or point pairs) actually computed */
  int64_t cells_unpruned; /* DP cells (or point pairs) of all pairs, in band */
  int64_t rescored;       /* pairs re-scored with compensated FP32 */
  int64_t rescored_fp64;  /* of those, pairs also re-scored in FP64 (near-ties) */
  int32_t launches;       /* kernels launched (graph replays count their nodes) */
  int32_t graph_replay;   /* 1 when the call replayed a captured graph */
} tsim_stats;

/* stages timed when profiling is on (tsim_ctx_set_profiling) */
typedef enum tsim_stage {
  TSIM_STAGE_SUMMARY = 0, /* query summaries */
  TSIM_STAGE_LB1,         /* O(1) bounds of all pairs */
  TSIM_STAGE_SEED,        /* seed selection + seed refinement */
  TSIM_STAGE_FILTER,      /* threshold, compaction, O(length) bounds, scan */
  TSIM_STAGE_DP,          /* exact FP32 DP / distance of round 1 (best by bound) */
  TSIM_STAGE_SELECT,      /* k-th value and re-score set */
  TSIM_STAGE_RESCORE,     /* compensated / FP64 re-score and final sort */
  TSIM_STAGE_REF,         /* reference-semantics batch calls */
  TSIM_STAGE_DP_SURVIVORS, /* exact FP32 DP of the pairs left after round 1 */
  TSIM_STAGE_COUNT
} tsim_stage;

typedef struct tsim_ctx tsim_ctx; /* device, stream, scratch, tuning cache */
typedef struct tsim_db tsim_db;   /* device-resident candidate set + summaries */

TSIM_API const char* tsim_status_string(int status);
TSIM_API const char* tsim_last_error(void);
TSIM_API int tsim_version(void);

/* ---- context ------------------------------------------------------------ */
/* Threads: a context, and the databases created on it, serve one thread at a
 * time (the caller serialises calls on one context; separate contexts run
 * concurrently).  A server's submit and wait may be called from any number
 * of threads, and the reference-named entry points serialise themselves on
 * their shared context.
 * stream: a cudaStream_t, or NULL for a stream the context creates. */
TSIM_API int tsim_ctx_create(int device, void* stream, tsim_ctx** out);
TSIM_API int tsim_ctx_destroy(tsim_ctx* ctx);
TSIM_API int tsim_ctx_set_stream(tsim_ctx* ctx, void* stream);
TSIM_API int tsim_ctx_synchronize(tsim_ctx* ctx);
/* bytes of device scratch the context currently holds */
TSIM_API int64_t tsim_ctx_scratch_bytes(const tsim_ctx* ctx);
/* Per-stage CUDA-event timing on the context stream (off by default). */
TSIM_API int tsim_ctx_set_profiling(tsim_ctx* ctx, int on);
/* Accumulated stage times (ms[TSIM_STAGE_COUNT], calls[TSIM_STAGE_COUNT]) and
 * the number of kernels this context launched; synchronises the stream.
 * reset != 0 clears the counters after reading. */
TSIM_API int tsim_ctx_counters(tsim_ctx* ctx, double* ms, int64_t* calls, int64_t* launches,
                               int64_t* dp_cells, int reset);
/* Number of streams one kNN request may use (default 4): the queries are
 * split into chunks run concurrently on internal child streams, forked from
 * and joined back to the context stream, so that latency-bound stages of
 * different chunks overlap.  1 runs everything on the context stream. */
TSIM_API int tsim_ctx_set_concurrency(tsim_ctx* ctx, int streams);
/* DP cells computed by the survivor round (TSIM_STAGE_DP_SURVIVORS) since the
 * last counter reset (synchronises). */
TSIM_API int tsim_ctx_survivor_cells(tsim_ctx* ctx, int64_t* cells);
/* Measured FP32 FMA throughput of this GPU in TFLOP/s (a short probe kernel,
 * for roofline denominators). */
TSIM_API int tsim_probe_fp32_tflops(tsim_ctx* ctx, double* tflops);

/* ---- debugging hooks (no counterpart in the reference, whose host code exits
 * on the first CUDA error: CudaRuntime1/common.cuh CHECK) ------------------ */
/* After `skip` more device or pinned-host allocations of the library succeed,
 * the next `count` fail as if the GPU were out of memory: the call that meets
 * one returns TSIM_ERR_OUT_OF_MEMORY and leaves its context usable.  count 0
 * disarms.  Process-wide; for tests of the error paths. */
TSIM_API int tsim_debug_fail_allocations(int skip, int count);
/* on != 0: every call fills the scratch it reserves with 0xff bytes (NaN
 * floats, -1 integers) before its kernels run, so a kernel that reads scratch
 * before writing it changes results.  Process-wide; slows every call. */
TSIM_API int tsim_debug_set_canary(int on);
/* Attempts of the device-side bounded waits (a kernel waiting for its bulk
 * copies of candidate points): attempts < 0 restores the default (about 4 M,
 * seconds at most); 0 makes every such wait run out at once.  A wait that
 * runs out sets the context's status word, the kernel reads the points from
 * global memory instead (results unchanged) and waits for its copies before
 * it exits; the next synchronising call (stats requested, or the
 * host-pointer entry point) returns TSIM_ERR_TIMEOUT and clears the word.
 * Process-wide; for tests of the timeout path. */
TSIM_API int tsim_debug_set_wait_limit(int64_t attempts);
/* libtsim_debug.so (built with TSIM_DEBUG_BOUNDS): every shared-memory index
 * of the DP and pairwise kernels is checked; one outside its array is
 * replaced by 0 (the kernel carries on, touching nothing outside) and
 * counted.  *count = violations since load, *first = (index << 32) | array
 * size of the first (may be NULL); *count = -1 in the product library,
 * which has no checks. */
TSIM_API int tsim_debug_bounds_violations(int64_t* count, int64_t* first);

/* ---- device-resident candidate database ---------------------------------- */
/* Copies host points/offsets to the device and builds per-trajectory
 * summaries (bounding box, first/last point).  Offsets start at 0 and
 * increase (no empty trajectory, none over 2^31 - 1 points); host_pts may be
 * NULL only when count is 0.  TSIM_ERR_INVALID_ARG otherwise. */
TSIM_API int tsim_db_create(tsim_ctx* ctx, const tsim_point* host_pts, const int64_t* host_off,
                            int count, tsim_db** out);
/* Wraps device-resident points/offsets (not copied, caller keeps them alive).
 * max_len is advisory: the longest trajectory is taken from the offsets.
 * On a database larger than L2, DTW's LB_Keogh stage fetches candidate
 * points by bulk copy when dev_pts is 16-byte aligned (cudaMalloc's 256-byte
 * alignment is; an offset into a larger allocation may not be), else with
 * ordinary loads: the results are the same either way. */
TSIM_API int tsim_db_wrap_device(tsim_ctx* ctx, const tsim_point* dev_pts,
                                 const int64_t* dev_off, int count, int max_len, tsim_db** out);
TSIM_API int tsim_db_destroy(tsim_db* db);
/* On-disk form of a database: points, offsets and the resident summaries in
 * one flat little-endian file with a checksum; loading copies it straight
 * into device memory (no summary rebuild).  Corrupt, truncated or foreign
 * files are refused. */
TSIM_API int tsim_db_save(const tsim_db* db, const char* path);
TSIM_API int tsim_db_load(tsim_ctx* ctx, const char* path, tsim_db** out);
TSIM_API int tsim_db_count(const tsim_db* db);
TSIM_API int64_t tsim_db_device_bytes(const tsim_db* db);

/* ---- exact kNN ------------------------------------------------------------ */
/* Cells inside the DP band (DTW, LCSS window, Frechet: n*m) summed over all
 * query x database pairs: the unpruned work, for "effective" cell rates. */
TSIM_API int tsim_band_cells(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                             const int64_t* d_qoff, int nq, tsim_db* db, int64_t* cells);
/* Device pointers; results d_ids[nq*k], d_dists[nq*k] (float), d_dists64
 * optional (may be NULL): DTW's compensated FP32 value (FP32 cell costs, path
 * sum compensated: within 4 2^-24 + O(P 2^-48) relative of FP64); Frechet's
 * and Hausdorff's FP32 value (one rounded cost, within 8 2^-24); Euclidean's compensated FP32 sum (or FP64 beyond 1024
 * points); the FP64 value for near-tied pairs and with
 * TSIM_FLAG_FP64_RESCORE.  Ids are exact in every case.  LCSS distances are
 * the integer match counts.  Asynchronous on the context stream unless stats
 * is non-NULL (then the call synchronises to fill it). */
TSIM_API int tsim_knn(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                      const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int* d_ids,
                      float* d_dists, double* d_dists64, tsim_stats* stats);
/* Host pointers end to end: copies the queries in and the results out
 * through the context's pinned and device staging buffers (kept between
 * calls, grown on demand, freed by tsim_ctx_destroy); synchronous. */
TSIM_API int tsim_knn_host(tsim_ctx* ctx, const tsim_params* p, const tsim_point* h_qpts,
                           const int64_t* h_qoff, int nq, tsim_db* db, int* h_ids,
                           float* h_dists, tsim_stats* stats);

/* ---- autotuner --------------------------------------------------------------
 * Times the launch choices of the exact kNN path on the caller's request
 * (first rows per lane-group of the anti-diagonal DP's passes: 1 .. 16, or
 * 0 = striped kernel only; concurrent query chunks: 1, 2, 4, 8) and records the fastest
 * for the request's shape class (measure, cost, band, window, k, log2 of the
 * longest query, the longest candidate, the database size and the query
 * count).  Later tsim_knn calls of that class use it.  Results never depend
 * on the choices.  The table is per context; save/load keep it in a text
 * file tagged with the device name (loading a file of another device fails). */
typedef struct tsim_tune_result {
  int rdiag;         /* chosen rows per lane-group (0: striped kernel only, -1: n/a) */
  int streams;       /* chosen concurrent query chunks */
  double best_ms;    /* median time of the chosen configuration */
  double default_ms; /* median time of the untuned defaults */
  int tried;         /* configurations timed */
} tsim_tune_result;
TSIM_API int tsim_autotune(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                           const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int reps,
                           tsim_tune_result* out);
TSIM_API int tsim_tuning_save(tsim_ctx* ctx, const char* path);
TSIM_API int tsim_tuning_load(tsim_ctx* ctx, const char* path);
TSIM_API int tsim_tuning_clear(tsim_ctx* ctx);
TSIM_API int tsim_tuning_count(const tsim_ctx* ctx);

/* Device scratch one tsim_knn call of this shape takes (per query chunk;
 * the server admits requests against it). */
TSIM_API int64_t tsim_knn_scratch_bytes(const tsim_params* p, int nq, int max_qlen,
                                        const tsim_db* db);

/* ---- Serving loop: continuous batching of kNN requests -----------------
 * A server owns `slots` device streams and one device pool of
 * `hbm_budget_bytes`.  Submitted requests (any measure, any query lengths)
 * wait in a FIFO queue; a worker thread admits the head request as soon as a
 * slot is free and its scratch (tsim_knn_scratch_bytes + staging) fits in the
 * pool, so requests that arrive while others run start at once and their
 * kernels overlap on the GPU.  The database stays resident.  A request's
 * results do not depend on what else is in flight.  The streams of the slots
 * share the process's hardware work queues: set CUDA_DEVICE_MAX_CONNECTIONS
 * (default 8, at most 32) to the slot count before CUDA initialises. */
typedef struct tsim_server tsim_server;
typedef struct tsim_server_opts {
  int slots;                /* requests in flight at once (0: 16) */
  int64_t hbm_budget_bytes; /* device pool for requests in flight (0: 1 GiB) */
  int queue_cap;            /* requests waiting for admission (0: 65536) */
} tsim_server_opts;
typedef struct tsim_request_info {
  int status;             /* tsim_status of the request */
  int nq, k;
  double queue_ms;        /* submit -> admission (host clock) */
  double latency_ms;      /* submit -> results ready on the host (host clock) */
  double device_ms;       /* CUDA-event time of the request on its stream */
  int64_t scratch_bytes;  /* device memory it was admitted with */
  int inflight_at_admit;  /* other requests on the device when it was admitted */
} tsim_request_info;
typedef struct tsim_server_stats {
  int64_t submitted, completed, failed, rejected;
  int queued, in_flight, peak_in_flight, slots;
  int64_t budget_bytes, scratch_in_use, peak_scratch_bytes;
  double launch_ms;   /* host time the worker spent enqueueing requests */
  double busy_ms;     /* host time the worker spent on anything but waiting */
  int64_t shared_threshold_hits; /* queries that started from an earlier identical query's
                                    threshold (TSIM_FLAG_SHARE_THRESHOLDS) */
} tsim_server_stats;

TSIM_API int tsim_server_create(tsim_ctx* ctx, tsim_db* db, const tsim_server_opts* opts,
                                tsim_server** out);
/* Copies the query (host CSR, h_qoff[0] == 0) and returns at once with a
 * ticket; TSIM_ERR_BUSY when the queue is full, TSIM_ERR_BUDGET when the
 * request could never fit the pool. */
TSIM_API int tsim_server_submit(tsim_server* s, const tsim_params* p, const tsim_point* h_qpts,
                                const int64_t* h_qoff, int nq, uint64_t* ticket);
/* Waits up to timeout_ms (< 0: forever) for a request; on completion copies
 * h_ids[nq*k], h_dists[nq*k] (either may be NULL), fills info (may be NULL),
 * forgets the ticket and returns the request's status.  TSIM_PENDING if it
 * is still running. */
TSIM_API int tsim_server_wait(tsim_server* s, uint64_t ticket, int timeout_ms, int* h_ids,
                              float* h_dists, tsim_request_info* info);
TSIM_API int tsim_server_get_stats(tsim_server* s, tsim_server_stats* st);
/* Finishes the requests in flight, fails the queued ones, frees the pool. */
TSIM_API int tsim_server_destroy(tsim_server* s);

/* Values of given (query, candidate) pairs -- d_pairs[2*i] = query index,
 * d_pairs[2*i+1] = candidate index -- for DTW, LCSS or Frechet under p's
 * band / window / cost.  precision: 0 = FP32 (d_out32), 1 = compensated FP32
 * (d_out64), 2 = FP64 (d_out64).  kernel: 0 = automatic, 1 = round-striped
 * DP, 2 = anti-diagonal DP with a warp per pair, 3 = with a CTA of 8 warps
 * per pair, 4 = with 2 warps per pair (pairs they cannot take fall back to 1),
 * 5 = a lane per pair (FP32 DTW, Frechet and LCSS, the throughput form for
 * many pairs; pairs whose band is too wide for it, and the other precisions,
 * go to 2, then 1), 6 = band-relative anti-diagonal with a warp per pair
 * (DTW and Frechet; lanes hold the live cells of an anti-diagonal; pairs
 * with more than 64 per anti-diagonal go to 2, then 1).  Every kernel
 * computes the same cells with the same operations.  Frechet
 * values are squared distances; LCSS values are match counts. */
TSIM_API int tsim_dp_pairs(tsim_ctx* ctx, const tsim_params* p, int precision, int kernel,
                           const tsim_point* d_qpts, const int64_t* d_qoff, int max_qlen,
                           const tsim_point* d_cpts, const int64_t* d_coff, int max_clen,
                           const int* d_pairs, int npairs, float* d_out32, double* d_out64);

/* ---- reference-semantics batch calls (device pointers) -------------------- */
/* DTW (Euclidean cell cost), LCSS (count/min(n,m)), Frechet: num_t queries of
 * length n against num_t candidates of length m, out[num_t].  The r=5
 * envelope bound ranks all candidates, the K=min(10,num_t) best by (bound,
 * index) (LCSS: bound descending, then index) are refined exactly, out[i] is
 * the best refined value (CudaRuntime1/dtw.cpp:14-113, lcss.cpp:13-115,
 * frechet.cpp:13-124). */
TSIM_API int tsim_ref_batch(tsim_ctx* ctx, int measure, const tsim_point* d_t1,
                            const tsim_point* d_t2, int num_t, int n, int m, float epsilon,
                            float* d_out);
/* Bytes of device memory that the scratch array of tsim_ref_batch_static
 * occupies on every GPU that loads libtsim.so, until the process exits. */
#define TSIM_STATIC_SCRATCH_BYTES (4u << 20)
/* No counterpart in the reference.  tsim_ref_batch for callers that may not
 * allocate device memory -- e.g. a plugin inside a host application that owns
 * the whole GPU memory pool, or a latency-critical loop that cannot take the
 * implicit synchronisation of cudaMalloc/cudaFree.  Same inputs, outputs and
 * results as tsim_ref_batch, on the caller's stream (NULL = legacy default
 * stream), with no context and no cudaMalloc/cudaFree: scratch comes from a
 * fixed array of TSIM_STATIC_SCRATCH_BYTES in the library's device memory.
 * Limit: the candidate keys (8*num_t bytes) and envelopes (16*m bytes) must
 * fit in 200 KiB of shared memory, i.e. num_t <= 25600 - 2*m (the scratch
 * array, about 136*num_t bytes, is not the binding limit); larger calls
 * return TSIM_ERR_UNSUPPORTED.  The kernels run on the current device, and a
 * non-NULL stream must belong to it (TSIM_ERR_INVALID_ARG otherwise).
 * The first call in each CUDA context (per device: the runtime's primary
 * context, or a driver-API context the caller made current; again after a
 * cudaDeviceReset) looks up the array's device address in that context
 * (cudaGetSymbolAddress) and caches it by the context's unique id; make that
 * first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race, so the caller serialises them (one stream,
 * or its own lock).  The array keeps the last call's contents; nothing in it
 * needs clearing, as every entry read is written earlier in the same call. */
TSIM_API int tsim_ref_batch_static(int measure, const tsim_point* d_t1, const tsim_point* d_t2,
                                   int num_t, int n, int m, float epsilon, float* d_out,
                                   void* stream);
/* Min over the given candidates of the symmetric Hausdorff distance
 * (CudaRuntime1/hausdorff.cu:84-122). d_cand[num_t1*top_k]. */
TSIM_API int tsim_hausdorff_cands(tsim_ctx* ctx, const tsim_point* d_t1, int num_t1, int n,
                                  const tsim_point* d_t2, int num_t2, int m, const int* d_cand,
                                  int top_k, float* d_out);
/* Min over CSR candidates of the lock-step Euclidean distance
 * (CudaRuntime1/euclidean.cu:17-73); bit-identical to the FP64 CPU path
 * (euclidean.cpp:27-40): FP32 compensated sums rank, FP64 re-scores. */
TSIM_API int tsim_euclid_cands(tsim_ctx* ctx, const tsim_point* d_t1, const tsim_point* d_t2,
                               const int* d_cand, const int* d_off, int num_t, int n,
                               int total_candidates, float* d_out);
/* Bounding-box nearest neighbours, the candidate generator that replaces the
 * reference's Boost R-tree query (hausdorff_rtree.cpp:38-69,
 * euclidean_rtree.cpp:49-69): the k nearest boxes by squared box-box
 * distance, ties by index, padded with the last one when num_t2 < k. */
TSIM_API int tsim_mbr_knn(tsim_ctx* ctx, const tsim_point* d_t1, int num_t1, int n,
                          const tsim_point* d_t2, int num_t2, int m, int k, int* d_out);

#ifdef __cplusplus
}
#endif
#endif
