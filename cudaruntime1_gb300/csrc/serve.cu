// serve.cu -- the serving loop: continuous batching of kNN requests over a
// device-resident database.
//
// The reference answers one synchronous batch per call and allocates, copies
// and frees per call (CudaRuntime1/dtw.cu:99-234 and its siblings).  Here a
// server keeps the database resident and owns:
//   * `slots` contexts, each with its own non-blocking stream: a request in a
//     slot runs the whole exact-kNN pipeline (knn.cu) on that stream, so
//     requests in different slots overlap on the GPU;
//   * one device pool of `hbm_budget_bytes`, carved first-fit: a request is
//     admitted with a block holding its staging (query points, offsets,
//     result ids and distances) and the scratch arena of its pipeline
//     (knn_scratch_bytes), lent to the slot context, which never grows it;
//   * a FIFO admission queue and one worker thread.  The worker admits the
//     head request as soon as a slot is free and its block fits the pool,
//     together with up to 15 queued requests of the same parameters (found
//     among the next 64): their queries run as one pipeline call, which
//     fills the GPU far better than single-query calls.  It polls the slots'
//     completion events; a request that arrives while others run starts as
//     soon as a slot and memory free up.
// A query's top-k depends only on that query and the read-only database (no
// stage couples the queries of a call), so results are the same alone, in
// a batch and in any mix.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tsim_internal.cuh"

namespace tsim {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  uint64_t ticket = 0;
  tsim_params p{};
  std::vector<tsim_point> pts;
  std::vector<int64_t> off;
  int nq = 0, max_qlen = 0, qb = 0;  // qb: queries per pipeline call
  size_t o_off = 0, o_ids = 0, o_dists = 0, staging = 0, scratch = 0;
  Clock::time_point t_submit, t_admit, t_done;
  int status = TSIM_PENDING;
  std::string error;
  std::vector<int> ids;
  std::vector<float> dists;
  float device_ms = 0.0f;
  int inflight_at_admit = 0;
  bool done = false;
};

// first fit over [0, size) (offsets and lengths in bytes, multiples of 256)
class Pool {
 public:
  void init(size_t n) {
    free_.clear();
    if (n) free_[0] = n;
  }
  bool alloc(size_t n, size_t& off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      off = it->first;
      const size_t rest = it->second - n, o2 = it->first + n;
      free_.erase(it);
      if (rest) free_[o2] = rest;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t n) {
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<size_t, size_t> free_;
};

// Requests admitted together into one slot: the same parameters, their
// queries concatenated into one pipeline call (continuous batching).  A
// query's top-k never depends on the other queries of its call.
constexpr int kMaxBatch = 16;     // requests per batch
constexpr int kLookahead = 64;    // queue entries scanned for batch mates

struct Slot {
  tsim_ctx* ctx = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr, done = nullptr;
  char* pinned = nullptr;
  size_t pinned_cap = 0;
  std::vector<Request*> batch;  // empty: the slot is free
  std::vector<int> first_q;     // each request's first query in the batch
  int nq = 0, max_qlen = 0, qb = 0;
  size_t o_off = 0, o_thr_in = 0, o_ids = 0, o_dists = 0, o_thr_out = 0, staging = 0, scratch = 0;
  size_t off = 0, bytes = 0;
  bool share = false;  // the batch shares pruning thresholds (TSIM_FLAG_SHARE_THRESHOLDS)
};

// Key of one query under one parameter set: the parameters that shape its
// answer and its points' bytes.
std::string share_key(const tsim_params& p, const tsim_point* pts, int64_t count) {
  std::string k;
  const int head[5] = {p.measure, p.k, p.cost, p.band_pct, p.delta};
  k.append(reinterpret_cast<const char*>(head), sizeof(head));
  k.append(reinterpret_cast<const char*>(&p.epsilon), sizeof(p.epsilon));
  k.append(reinterpret_cast<const char*>(pts), sizeof(tsim_point) * (size_t)count);
  return k;
}

bool same_params(const tsim_params& a, const tsim_params& b) {
  return a.measure == b.measure && a.k == b.k && a.cost == b.cost && a.band_pct == b.band_pct &&
         a.epsilon == b.epsilon && a.delta == b.delta && a.flags == b.flags;
}

}  // namespace
}  // namespace tsim

struct tsim_server {
  tsim_ctx* ctx = nullptr;
  tsim_db* db = nullptr;
  size_t budget = 0;
  int queue_cap = 0;
  char* pool_base = nullptr;
  tsim::Pool pool;
  std::vector<tsim::Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<tsim::Request*> queue;
  std::unordered_map<uint64_t, tsim::Request*> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  int64_t submitted = 0, completed = 0, failed = 0, rejected = 0;
  int in_flight = 0, peak_in_flight = 0;
  size_t in_use = 0, peak_in_use = 0;
  double launch_ms = 0.0, busy_ms = 0.0;
  // pruning thresholds of completed queries (TSIM_FLAG_SHARE_THRESHOLDS),
  // keyed by parameters and query points, oldest evicted first (worker only)
  std::unordered_map<std::string, float> shared;
  std::deque<std::string> shared_order;
  int64_t shared_hits = 0;
  std::thread worker;
};

namespace tsim {
namespace {

// Lay out a batch's staging (queries, offsets, ids, distances) and size its
// pipeline scratch.
constexpr size_t kSharedCap = 65536;  // queries whose thresholds the server keeps

void sl_hits(tsim_server* s, int hits) {
  std::lock_guard<std::mutex> g(s->mu);
  s->shared_hits += hits;
}

void plan_batch(tsim_server* s, Slot& sl) {
  const tsim_params& p = sl.batch[0]->p;
  sl.first_q.clear();
  sl.nq = 0;
  sl.max_qlen = 0;
  size_t npts = 0;
  for (Request* r : sl.batch) {
    sl.first_q.push_back(sl.nq);
    sl.nq += r->nq;
    sl.max_qlen = std::max(sl.max_qlen, r->max_qlen);
    npts += r->pts.size();
  }
  const int64_t kMaxPairs = int64_t(1) << 24;
  sl.qb = (int)std::max<int64_t>(1, std::min<int64_t>(sl.nq, kMaxPairs / std::max(s->db->count, 1)));
  sl.scratch = align256(knn_scratch_bytes(&p, sl.qb, sl.max_qlen, s->db));
  // staging: queries, offsets, shared thresholds in (copied to the device);
  // ids, distances, thresholds out (copied back)
  sl.share = (p.flags & TSIM_FLAG_SHARE_THRESHOLDS) != 0;
  sl.o_off = align256(sizeof(tsim_point) * npts);
  sl.o_thr_in = sl.o_off + align256(sizeof(int64_t) * (sl.nq + 1));
  sl.o_ids = sl.o_thr_in + (sl.share ? align256(sizeof(float) * sl.nq) : 0);
  sl.o_dists = sl.o_ids + align256(sizeof(int) * (size_t)sl.nq * p.k);
  sl.o_thr_out = sl.o_dists + align256(sizeof(float) * (size_t)sl.nq * p.k);
  sl.staging = sl.o_thr_out + (sl.share ? align256(sizeof(float) * sl.nq) : 0);
  sl.bytes = sl.staging + sl.scratch;
}

// Enqueue the batch's work on its slot's stream (no lock held).
int launch(tsim_server* s, Slot& sl) {
  tsim_ctx* c = sl.ctx;
  char* base = s->pool_base + sl.off;
  if (sl.pinned_cap < sl.staging) {  // the slot is idle: nothing reads the old buffer
    if (sl.pinned) TSIM_CUDA(cudaFreeHost(sl.pinned));
    sl.pinned = nullptr;
    sl.pinned_cap = 0;
    const size_t cap = std::max<size_t>(sl.staging, size_t(1) << 20);
    TSIM_CUDA(host_alloc((void**)&sl.pinned, cap));
    sl.pinned_cap = cap;
  }
  // concatenate the queries and rebase their offsets
  int64_t* hoff = reinterpret_cast<int64_t*>(sl.pinned + sl.o_off);
  size_t pt = 0;
  int qi = 0;
  hoff[0] = 0;
  float* hthr = reinterpret_cast<float*>(sl.pinned + sl.o_thr_in);
  int hits = 0;
  for (Request* r : sl.batch) {
    memcpy(sl.pinned + sizeof(tsim_point) * pt, r->pts.data(), sizeof(tsim_point) * r->pts.size());
    for (int i = 0; i < r->nq; ++i) {
      hoff[qi + i + 1] = (int64_t)pt + r->off[i + 1];
      if (sl.share) {  // an earlier identical query's threshold, else none
        const auto it = s->shared.find(share_key(r->p, r->pts.data() + r->off[i],
                                                 r->off[i + 1] - r->off[i]));
        const bool hit = it != s->shared.end();
        hits += hit;
        hthr[qi + i] = hit ? it->second : (r->p.measure == TSIM_LCSS ? 0.0f : HUGE_VALF);
      }
    }
    pt += r->pts.size();
    qi += r->nq;
  }
  sl_hits(s, hits);
  TSIM_CUDA(cudaMemcpyAsync(base, sl.pinned, sl.o_ids, cudaMemcpyHostToDevice, c->stream));
  c->arena = base + sl.staging;
  c->arena_cap = sl.scratch;
  c->arena_used = 0;
  TSIM_CUDA(cudaEventRecord(sl.t0, c->stream));
  const tsim_params& p = sl.batch[0]->p;
  const float2* qpts = reinterpret_cast<const float2*>(base);
  const int64_t* qoff = reinterpret_cast<const int64_t*>(base + sl.o_off);
  int* ids = reinterpret_cast<int*>(base + sl.o_ids);
  float* dists = reinterpret_cast<float*>(base + sl.o_dists);
  const int k = p.k;
  const float* thr_in = sl.share ? reinterpret_cast<const float*>(base + sl.o_thr_in) : nullptr;
  float* thr_out = sl.share ? reinterpret_cast<float*>(base + sl.o_thr_out) : nullptr;
  for (int q0 = 0; q0 < sl.nq; q0 += sl.qb) {
    const int nb = std::min(sl.qb, sl.nq - q0);
    TSIM_TRY(knn(c, &p, qpts, qoff + q0, nb, sl.max_qlen, s->db, ids + (size_t)q0 * k,
                 dists + (size_t)q0 * k, nullptr, nullptr, thr_in ? thr_in + q0 : nullptr,
                 thr_out ? thr_out + q0 : nullptr));
  }
  TSIM_CUDA(cudaEventRecord(sl.t1, c->stream));
  TSIM_CUDA(cudaMemcpyAsync(sl.pinned + sl.o_ids, base + sl.o_ids, sl.staging - sl.o_ids,
                            cudaMemcpyDeviceToHost, c->stream));
  TSIM_CUDA(cudaEventRecord(sl.done, c->stream));
  return TSIM_OK;
}

// Retire the slot's batch (lock held; its stream work has ended).
void finish(tsim_server* s, Slot& sl, int status, const std::string& err) {
  float dms = 0.0f;
  if (status == TSIM_OK && cudaEventElapsedTime(&dms, sl.t0, sl.t1) != cudaSuccess) dms = 0.0f;
  const Clock::time_point now = Clock::now();
  for (size_t b = 0; b < sl.batch.size(); ++b) {
    Request* r = sl.batch[b];
    if (status == TSIM_OK) {
      const size_t nk = (size_t)r->nq * r->p.k, at = (size_t)sl.first_q[b] * r->p.k;
      r->ids.resize(nk);
      r->dists.resize(nk);
      memcpy(r->ids.data(), sl.pinned + sl.o_ids + sizeof(int) * at, sizeof(int) * nk);
      memcpy(r->dists.data(), sl.pinned + sl.o_dists + sizeof(float) * at, sizeof(float) * nk);
      r->device_ms = dms;
      ++s->completed;
      if (sl.share) {  // the queries' final thresholds, for later identical queries
        const float* t = reinterpret_cast<const float*>(sl.pinned + sl.o_thr_out) + sl.first_q[b];
        for (int i = 0; i < r->nq; ++i) {
          std::string key = share_key(r->p, r->pts.data() + r->off[i], r->off[i + 1] - r->off[i]);
          auto it = s->shared.find(key);
          if (it != s->shared.end()) {
            it->second = r->p.measure == TSIM_LCSS ? std::max(it->second, t[i])
                                                   : std::min(it->second, t[i]);
            continue;
          }
          if (s->shared_order.size() >= kSharedCap) {  // evict the oldest
            s->shared.erase(s->shared_order.front());
            s->shared_order.pop_front();
          }
          s->shared_order.push_back(key);
          s->shared.emplace(std::move(key), t[i]);
        }
      }
    } else {
      r->error = err;
      ++s->failed;
    }
    r->status = status;
    r->t_done = now;
    r->done = true;
  }
  s->pool.release(sl.off, sl.bytes);
  s->in_use -= sl.bytes;
  s->in_flight -= (int)sl.batch.size();
  sl.batch.clear();
  sl.ctx->arena = nullptr;
  sl.ctx->arena_cap = 0;
  s->cv_done.notify_all();
}

void worker_loop(tsim_server* s) {
  cudaSetDevice(s->ctx->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    const Clock::time_point t_round = Clock::now();
    bool progressed = false;
    for (Slot& sl : s->slots) {  // completions
      if (sl.batch.empty()) continue;
      const cudaError_t e = cudaEventQuery(sl.done);
      if (e == cudaErrorNotReady) continue;
      if (e == cudaSuccess)
        finish(s, sl, TSIM_OK, "");
      else
        finish(s, sl, TSIM_ERR_CUDA, std::string("request failed on the device: ") +
                                         cudaGetErrorString(e));
      progressed = true;
    }
    while (!s->queue.empty()) {  // admissions: the head request and its batch mates
      Slot* sl = nullptr;
      for (Slot& x : s->slots)
        if (x.batch.empty()) {
          sl = &x;
          break;
        }
      if (!sl) break;
      Request* r0 = s->queue.front();
      std::vector<size_t> picked{0};  // queue positions of the batch
      sl->batch.assign(1, r0);
      for (size_t qi = 1; qi < s->queue.size() && qi < (size_t)kLookahead &&
                          sl->batch.size() < (size_t)kMaxBatch;
           ++qi)
        if (same_params(s->queue[qi]->p, r0->p)) {
          picked.push_back(qi);
          sl->batch.push_back(s->queue[qi]);
        }
      plan_batch(s, *sl);
      size_t off = 0;
      bool fits = s->pool.alloc(sl->bytes, off);
      if (!fits && sl->batch.size() > 1) {
        picked.resize(1);  // the batch does not fit: the head request alone
        sl->batch.resize(1);
        plan_batch(s, *sl);
        fits = s->pool.alloc(sl->bytes, off);
      }
      if (!fits) {
        sl->batch.clear();
        break;  // waits for memory to free up
      }
      for (size_t i = picked.size(); i-- > 0;) s->queue.erase(s->queue.begin() + picked[i]);
      sl->off = off;
      const Clock::time_point now = Clock::now();
      for (Request* r : sl->batch) {
        r->t_admit = now;
        r->inflight_at_admit = s->in_flight;
      }
      s->in_flight += (int)sl->batch.size();
      s->peak_in_flight = std::max(s->peak_in_flight, s->in_flight);
      s->in_use += sl->bytes;
      s->peak_in_use = std::max(s->peak_in_use, s->in_use);
      lk.unlock();
      const Clock::time_point t0 = Clock::now();
      const int st = launch(s, *sl);
      const double lms = ms_between(t0, Clock::now());
      std::string err;
      if (st != TSIM_OK) {
        err = tsim_last_error();
        cudaStreamSynchronize(sl->ctx->stream);  // what was enqueued must end before the block is reused
      }
      lk.lock();
      s->launch_ms += lms;
      if (st != TSIM_OK) finish(s, *sl, st, err);
      progressed = true;
    }
    s->busy_ms += ms_between(t_round, Clock::now());
    if (s->stop && s->queue.empty() && s->in_flight == 0) break;
    if (!progressed) {
      if (s->in_flight == 0)
        s->cv_work.wait(lk);  // woken by a submit or by destroy
      else
        s->cv_work.wait_for(lk, std::chrono::microseconds(20));  // poll the slots
    }
  }
}

void server_free(tsim_server* s) {
  for (Slot& sl : s->slots) {
    if (sl.ctx) {
      sl.ctx->arena = nullptr;
      sl.ctx->arena_cap = 0;
      tsim_ctx_destroy(sl.ctx);
    }
    if (sl.t0) cudaEventDestroy(sl.t0);
    if (sl.t1) cudaEventDestroy(sl.t1);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.pinned) cudaFreeHost(sl.pinned);
  }
  if (s->pool_base) cudaFree(s->pool_base);
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
}

}  // namespace
}  // namespace tsim

using namespace tsim;

extern "C" int64_t tsim_knn_scratch_bytes(const tsim_params* p, int nq, int max_qlen,
                                          const tsim_db* db) {
  if (!p || !db || nq < 1 || max_qlen < 1 || db->count < 1 || p->k < 1) return -1;
  return (int64_t)knn_scratch_bytes(p, nq, max_qlen, db);
}

extern "C" int tsim_server_create(tsim_ctx* ctx, tsim_db* db, const tsim_server_opts* opts,
                                  tsim_server** out) {
  TSIM_CHECK_ARG(ctx && db && out, "NULL argument");
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  *out = nullptr;
  const int nslots = opts && opts->slots > 0 ? opts->slots : 16;
  const int64_t budget = opts && opts->hbm_budget_bytes > 0 ? opts->hbm_budget_bytes : int64_t(1) << 30;
  TSIM_CHECK_ARG(nslots <= 256, "at most 256 slots");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  tsim_server* s = new tsim_server;
  s->ctx = ctx;
  s->db = db;
  s->budget = (size_t)budget & ~size_t(255);
  s->queue_cap = opts && opts->queue_cap > 0 ? opts->queue_cap : 65536;
  s->slots.resize(nslots);
  int st = TSIM_OK;
  cudaError_t e = dev_malloc((void**)&s->pool_base, s->budget);
  if (e != cudaSuccess) st = cuda_fail(e, "server pool", __FILE__, __LINE__);
  for (int i = 0; i < nslots && st == TSIM_OK; ++i) {
    Slot& sl = s->slots[i];
    st = tsim_ctx_create(ctx->device, nullptr, &sl.ctx);
    if (st != TSIM_OK) break;
    sl.ctx->concurrency = 1;
    sl.ctx->arena_external = true;
    e = cudaEventCreate(&sl.t0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.t1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e != cudaSuccess) st = cuda_fail(e, "server events", __FILE__, __LINE__);
  }
  if (st != TSIM_OK) {
    server_free(s);
    return st;
  }
  s->pool.init(s->budget);
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return TSIM_OK;
}

extern "C" int tsim_server_submit(tsim_server* s, const tsim_params* p, const tsim_point* h_qpts,
                                  const int64_t* h_qoff, int nq, uint64_t* ticket) {
  TSIM_CHECK_ARG(s && p && h_qpts && h_qoff && ticket, "NULL argument");
  TSIM_CHECK_ARG(nq >= 1 && h_qoff[0] == 0, "nq must be >= 1 and offsets start at 0");
  TSIM_CHECK_ARG(p->k >= 1 && p->k <= 64, "k must be in 1..64");
  TSIM_CHECK_ARG(p->measure >= TSIM_DTW && p->measure <= TSIM_EUCLIDEAN, "unknown measure");
  TSIM_CHECK_ARG(p->measure != TSIM_LCSS || p->epsilon >= 0.0f, "LCSS epsilon must be >= 0");
  Request* r = new Request;
  r->p = *p;
  r->p.flags |= TSIM_FLAG_NO_GRAPH;
  r->nq = nq;
  for (int i = 0; i < nq; ++i) {
    if (h_qoff[i + 1] <= h_qoff[i]) {
      delete r;
      return fail(TSIM_ERR_INVALID_ARG, "queries must be non-empty");
    }
    r->max_qlen = std::max<int>(r->max_qlen, (int)(h_qoff[i + 1] - h_qoff[i]));
  }
  const size_t npts = (size_t)h_qoff[nq];
  r->pts.assign(h_qpts, h_qpts + npts);
  r->off.assign(h_qoff, h_qoff + nq + 1);
  const int64_t kMaxPairs = int64_t(1) << 24;
  r->qb = (int)std::max<int64_t>(1, std::min<int64_t>(nq, kMaxPairs / std::max(s->db->count, 1)));
  r->scratch = align256(knn_scratch_bytes(&r->p, r->qb, r->max_qlen, s->db));
  r->o_off = align256(sizeof(tsim_point) * npts);
  r->o_ids = r->o_off + align256(sizeof(int64_t) * (nq + 1));
  r->o_dists = r->o_ids + align256(sizeof(int) * (size_t)nq * p->k);
  r->staging = r->o_dists + align256(sizeof(float) * (size_t)nq * p->k);
  if (r->staging + r->scratch > s->budget) {
    const size_t need = r->staging + r->scratch;
    delete r;
    std::lock_guard<std::mutex> g(s->mu);
    ++s->rejected;
    return fail(TSIM_ERR_BUDGET, "request needs " + std::to_string(need) +
                                     " bytes of device memory, more than the server's pool");
  }
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop || (int)s->queue.size() >= s->queue_cap) {
      ++s->rejected;
      delete r;
      return fail(TSIM_ERR_BUSY, s->stop ? "server is stopping" : "admission queue full");
    }
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    ++s->submitted;
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return TSIM_OK;
}

extern "C" int tsim_server_wait(tsim_server* s, uint64_t ticket, int timeout_ms, int* h_ids,
                                float* h_dists, tsim_request_info* info) {
  TSIM_CHECK_ARG(s != nullptr, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  TSIM_CHECK_ARG(it != s->reqs.end(), "unknown ticket (never issued or already collected)");
  Request* r = it->second;
  if (timeout_ms < 0)
    s->cv_done.wait(lk, [r] { return r->done; });
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [r] { return r->done; }))
    return TSIM_PENDING;
  s->reqs.erase(it);
  lk.unlock();
  const size_t nk = (size_t)r->nq * r->p.k;
  if (r->status == TSIM_OK) {
    if (h_ids) memcpy(h_ids, r->ids.data(), sizeof(int) * nk);
    if (h_dists) memcpy(h_dists, r->dists.data(), sizeof(float) * nk);
  }
  if (info) {
    info->status = r->status;
    info->nq = r->nq;
    info->k = r->p.k;
    const bool admitted = r->t_admit.time_since_epoch().count() != 0;
    info->queue_ms = admitted ? ms_between(r->t_submit, r->t_admit) : ms_between(r->t_submit, r->t_done);
    info->latency_ms = ms_between(r->t_submit, r->t_done);
    info->device_ms = r->device_ms;
    info->scratch_bytes = (int64_t)(r->staging + r->scratch);
    info->inflight_at_admit = r->inflight_at_admit;
  }
  const int st = r->status;
  if (st != TSIM_OK) set_error(r->error);
  delete r;
  return st;
}

extern "C" int tsim_server_get_stats(tsim_server* s, tsim_server_stats* st) {
  TSIM_CHECK_ARG(s && st, "NULL argument");
  std::lock_guard<std::mutex> g(s->mu);
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->failed = s->failed;
  st->rejected = s->rejected;
  st->queued = (int)s->queue.size();
  st->in_flight = s->in_flight;
  st->peak_in_flight = s->peak_in_flight;
  st->slots = (int)s->slots.size();
  st->budget_bytes = (int64_t)s->budget;
  st->scratch_in_use = (int64_t)s->in_use;
  st->peak_scratch_bytes = (int64_t)s->peak_in_use;
  st->launch_ms = s->launch_ms;
  st->busy_ms = s->busy_ms;
  st->shared_threshold_hits = s->shared_hits;
  return TSIM_OK;
}

extern "C" int tsim_server_destroy(tsim_server* s) {
  if (!s) return TSIM_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (Request* r : s->queue) {  // never admitted
      r->status = TSIM_ERR_UNSUPPORTED;
      r->error = "server destroyed before the request was admitted";
      r->t_done = Clock::now();
      r->done = true;
      ++s->failed;
    }
    s->queue.clear();
    s->cv_done.notify_all();
  }
  s->cv_work.notify_one();
  if (s->worker.joinable()) s->worker.join();  // in-flight requests finish first
  server_free(s);
  return TSIM_OK;
}
