// capi.cu -- context, scratch arena, device-resident database and status
// reporting of the C ABI (include/tsim.h).
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <vector>

#include "debug_bounds.cuh"
#include "tsim_internal.cuh"

namespace tsim {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char b[512];
  snprintf(b, sizeof b, "%s failed at %s:%d: %s (%s)", what, file, line, cudaGetErrorName(e),
           cudaGetErrorString(e));
  g_last_error = b;
  return e == cudaErrorMemoryAllocation ? TSIM_ERR_OUT_OF_MEMORY : TSIM_ERR_CUDA;
}

// Allocation-failure injection (tsim_debug_fail_allocations): after `skip`
// more allocations succeed, the next `count` fail as out of memory.
std::atomic<long long> g_fail_skip{0};
std::atomic<long long> g_fail_count{0};
std::atomic<int> g_canary{0};

static bool injected_failure() {
  if (g_fail_count.load() <= 0) return false;
  if (g_fail_skip.fetch_sub(1) > 0) return false;
  return g_fail_count.fetch_sub(1) > 0;
}

cudaError_t dev_malloc(void** p, size_t bytes) {
  if (injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

cudaError_t host_alloc(void** p, size_t bytes) {
  if (injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

bool debug_canary() { return g_canary.load() != 0; }

// the bounds-check readers of the translation units (TSIM_DEBUG_BOUNDS
// build), registered during static initialisation
static std::vector<BoundsReader>& bounds_readers() {
  static std::vector<BoundsReader> v;
  return v;
}
int register_bounds_reader(BoundsReader r) {
  bounds_readers().push_back(r);
  return 0;
}

int arena_reserve(tsim_ctx* ctx, size_t bytes) {
  ctx->arena_used = 0;
  if (bytes <= ctx->arena_cap) {
    if (debug_canary() && bytes)
      TSIM_CUDA(cudaMemsetAsync(ctx->arena, 0xff, bytes, ctx->stream));
    return TSIM_OK;
  }
  if (ctx->arena_external)  // a block lent by a server: it never grows
    return fail(TSIM_ERR_BUDGET, "request needs more scratch than it was admitted with");
  size_t cap = std::max(bytes + bytes / 4, size_t(1) << 20);
  if (ctx->arena) {
    TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
    TSIM_CUDA(cudaFree(ctx->arena));
    ctx->arena = nullptr;
    ctx->arena_cap = 0;
  }
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&ctx->arena), cap));
  ctx->arena_cap = cap;
  ctx->arena_gen++;  // graphs captured over the old arena are stale
  if (debug_canary()) TSIM_CUDA(cudaMemsetAsync(ctx->arena, 0xff, bytes, ctx->stream));
  return TSIM_OK;
}

int pinned_reserve(tsim_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->pinned_cap) return TSIM_OK;
  size_t cap = std::max(bytes + bytes / 4, size_t(1) << 20);
  if (ctx->pinned) {
    TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
    TSIM_CUDA(cudaFreeHost(ctx->pinned));
    ctx->pinned = nullptr;
    ctx->pinned_cap = 0;
  }
  TSIM_CUDA(host_alloc(&ctx->pinned, cap));
  ctx->pinned_cap = cap;
  return TSIM_OK;
}

namespace {

// Per-trajectory summaries: bounding box and first/last point.
__global__ void summarize_kernel(const float2* __restrict__ pts, const int64_t* __restrict__ off,
                                 int count, float4* __restrict__ box, float4* __restrict__ ends,
                                 int* __restrict__ len) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = warp; t < count; t += nwarps) {
    const int64_t b = off[t], e = off[t + 1];
    float x0 = TSIM_INF, y0 = TSIM_INF, x1 = -TSIM_INF, y1 = -TSIM_INF;
    for (int64_t i = b + lane; i < e; i += 32) {
      float2 p = pts[i];
      x0 = fminf(x0, p.x);
      x1 = fmaxf(x1, p.x);
      y0 = fminf(y0, p.y);
      y1 = fmaxf(y1, p.y);
    }
    for (int o = 16; o; o >>= 1) {
      x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
      y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
      x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
      y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    if (lane == 0) {
      box[t] = make_float4(x0, y0, x1, y1);
      if (e > b) {
        float2 f = pts[b], l = pts[e - 1];
        ends[t] = make_float4(f.x, f.y, l.x, l.y);
      } else {
        ends[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      len[t] = (int)(e - b);
    }
  }
}

// Segment boxes and point sums: warp per trajectory, lane s < kSegs reduces
// segment s (sums in FP64, rounded once to float).
__global__ void segments_kernel(const float2* __restrict__ pts, const int64_t* __restrict__ off,
                                int count, float4* __restrict__ segbox, float2* __restrict__ segsum) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = warp; t < count; t += nwarps) {
    if (lane >= kSegs) continue;
    const int64_t b = off[t];
    const int m = (int)(off[t + 1] - b);
    const int s0 = (int)((long long)lane * m / kSegs), s1 = (int)((long long)(lane + 1) * m / kSegs);
    float x0 = TSIM_INF, y0 = TSIM_INF, x1 = -TSIM_INF, y1 = -TSIM_INF;
    double sx = 0.0, sy = 0.0;
    for (int j = s0; j < s1; ++j) {
      const float2 p = pts[b + j];
      x0 = fminf(x0, p.x);
      x1 = fmaxf(x1, p.x);
      y0 = fminf(y0, p.y);
      y1 = fmaxf(y1, p.y);
      sx += p.x;
      sy += p.y;
    }
    segbox[(size_t)t * kSegs + lane] = make_float4(x0, y0, x1, y1);
    segsum[(size_t)t * kSegs + lane] = make_float2((float)sx, (float)sy);
  }
}

}  // namespace

int summarize(tsim_ctx* ctx, const float2* pts, const int64_t* off, int count, float4* box,
              float4* ends, int* len) {
  if (count == 0) return TSIM_OK;
  int blocks = std::min((count + 7) / 8, ctx->num_sms * 16);
  summarize_kernel<<<blocks, 256, 0, ctx->stream>>>(pts, off, count, box, ends, len);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

int db_summarize(tsim_db* db) {
  if (db->count == 0) return TSIM_OK;
  int blocks = std::min((db->count + 7) / 8, db->ctx->num_sms * 16);
  summarize_kernel<<<blocks, 256, 0, db->ctx->stream>>>(db->pts, db->off, db->count, db->box,
                                                         db->ends, db->len);
  segments_kernel<<<blocks, 256, 0, db->ctx->stream>>>(db->pts, db->off, db->count, db->segbox,
                                                        db->segsum);
  TSIM_CUDA(cudaGetLastError());
  return TSIM_OK;
}

void stage_begin(tsim_ctx* ctx, int stage) {
  if (!ctx->profiling) return;
  if (ctx->nstage_ev >= 64) stage_collect(ctx);
  const int i = ctx->nstage_ev;
  for (int e = 2 * i; e < 2 * i + 2; ++e)
    if (!ctx->stage_ev[e]) cudaEventCreate(&ctx->stage_ev[e]);
  ctx->stage_id[i] = stage;
  cudaEventRecord(ctx->stage_ev[2 * i], ctx->stream);
}

void stage_end(tsim_ctx* ctx) {
  if (!ctx->profiling) return;
  cudaEventRecord(ctx->stage_ev[2 * ctx->nstage_ev + 1], ctx->stream);
  ctx->nstage_ev++;
}

int stage_collect(tsim_ctx* ctx) {
  if (ctx->nstage_ev == 0) return TSIM_OK;
  TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < ctx->nstage_ev; ++i) {
    float ms = 0.0f;
    TSIM_CUDA(cudaEventElapsedTime(&ms, ctx->stage_ev[2 * i], ctx->stage_ev[2 * i + 1]));
    ctx->stage_ms[ctx->stage_id[i]] += ms;
    ctx->stage_calls[ctx->stage_id[i]] += 1;
  }
  ctx->nstage_ev = 0;
  return TSIM_OK;
}

namespace {

// Independent FMA chains per thread; the result is stored so nothing is
// eliminated.  flops = 2 * kChains * iters per thread.
constexpr int kChains = 16;
__global__ void __launch_bounds__(256) fp32_probe_kernel(float* out, int iters, float a, float b) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = fmaf(v[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 123.456f) out[0] = s;
}

}  // namespace

}  // namespace tsim

using namespace tsim;

extern "C" int tsim_ctx_set_profiling(tsim_ctx* ctx, int on) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  if (!on) TSIM_TRY(stage_collect(ctx));
  ctx->profiling = on != 0;
  for (tsim_ctx* s : ctx->subs) {
    if (!on) TSIM_TRY(stage_collect(s));
    s->profiling = on != 0;
  }
  return TSIM_OK;
}

extern "C" int tsim_ctx_set_concurrency(tsim_ctx* ctx, int streams) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  TSIM_CHECK_ARG(streams >= 1 && streams <= 16, "streams must be in 1..16");
  ctx->concurrency = streams;
  return TSIM_OK;
}

namespace tsim {

// child contexts for concurrent chunks (created on first use)
int ensure_subs(tsim_ctx* ctx, int n) {
  if (!ctx->fork_ev) TSIM_CUDA(cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming));
  while ((int)ctx->subs.size() < n) {
    tsim_ctx* s = nullptr;
    TSIM_TRY(tsim_ctx_create(ctx->device, nullptr, &s));
    s->concurrency = 1;
    s->profiling = ctx->profiling;
    s->status = ctx->status;  // a chunk's timeouts are its request's
    ctx->subs.push_back(s);
    cudaEvent_t ev;
    TSIM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->join_ev.push_back(ev);
  }
  return TSIM_OK;
}

}  // namespace tsim

extern "C" int tsim_ctx_counters(tsim_ctx* ctx, double* ms, int64_t* calls, int64_t* launches,
                                 int64_t* dp_cells, int reset) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  double ms_acc[TSIM_STAGE_COUNT] = {};
  int64_t calls_acc[TSIM_STAGE_COUNT] = {};
  int64_t launches_acc = 0;
  unsigned long long cells_acc = 0;
  std::vector<tsim_ctx*> all{ctx};
  all.insert(all.end(), ctx->subs.begin(), ctx->subs.end());
  for (tsim_ctx* c : all) {  // the context and its child streams
    TSIM_TRY(stage_collect(c));
    TSIM_CUDA(cudaStreamSynchronize(c->stream));
    for (int s = 0; s < TSIM_STAGE_COUNT; ++s) {
      ms_acc[s] += c->stage_ms[s];
      calls_acc[s] += c->stage_calls[s];
    }
    launches_acc += c->launches;
    unsigned long long cells[2] = {0, 0};  // [0] all DP cells but [1] those of the survivor round
    TSIM_CUDA(cudaMemcpy(cells, c->dcounters, sizeof(cells), cudaMemcpyDeviceToHost));
    cells_acc += cells[0] + cells[1];
  }
  for (int s = 0; s < TSIM_STAGE_COUNT; ++s) {
    if (ms) ms[s] = ms_acc[s];
    if (calls) calls[s] = calls_acc[s];
  }
  if (launches) *launches = launches_acc;
  if (dp_cells) *dp_cells = (int64_t)cells_acc;
  if (reset)
    for (tsim_ctx* c : ctx->subs) {
      for (int s = 0; s < TSIM_STAGE_COUNT; ++s) {
        c->stage_ms[s] = 0.0;
        c->stage_calls[s] = 0;
      }
      c->launches = 0;
      TSIM_CUDA(cudaMemsetAsync(c->dcounters, 0, 64, c->stream));
      TSIM_CUDA(cudaStreamSynchronize(c->stream));
    }
  if (reset) {
    for (int s = 0; s < TSIM_STAGE_COUNT; ++s) {
      ctx->stage_ms[s] = 0.0;
      ctx->stage_calls[s] = 0;
    }
    ctx->launches = 0;
    TSIM_CUDA(cudaMemsetAsync(ctx->dcounters, 0, 64, ctx->stream));
    TSIM_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return TSIM_OK;
}

extern "C" int tsim_ctx_survivor_cells(tsim_ctx* ctx, int64_t* cells) {
  TSIM_CHECK_ARG(ctx && cells, "NULL argument");
  unsigned long long acc = 0;
  std::vector<tsim_ctx*> all{ctx};
  all.insert(all.end(), ctx->subs.begin(), ctx->subs.end());
  for (tsim_ctx* c : all) {
    TSIM_CUDA(cudaStreamSynchronize(c->stream));
    unsigned long long v = 0;
    TSIM_CUDA(cudaMemcpy(&v, c->dcounters + 1, sizeof(v), cudaMemcpyDeviceToHost));
    acc += v;
  }
  *cells = (int64_t)acc;
  return TSIM_OK;
}

extern "C" int tsim_debug_fail_allocations(int skip, int count) {
  TSIM_CHECK_ARG(skip >= 0 && count >= 0, "skip and count must be >= 0");
  tsim::g_fail_count.store(0);  // disarmed while the new values go in
  tsim::g_fail_skip.store(skip);
  tsim::g_fail_count.store(count);
  return TSIM_OK;
}

extern "C" int tsim_debug_bounds_violations(int64_t* count, int64_t* first) {
  TSIM_CHECK_ARG(count != nullptr, "count is NULL");
#ifdef TSIM_DEBUG_BOUNDS
  unsigned long long n = 0;
  long long f = 0;
  for (tsim::BoundsReader r : tsim::bounds_readers()) TSIM_CUDA(r(&n, &f));
  *count = (int64_t)n;
  if (first) *first = (int64_t)f;
#else
  *count = -1;  // built without the checks
  if (first) *first = 0;
#endif
  return TSIM_OK;
}

extern "C" int tsim_debug_set_canary(int on) {
  tsim::g_canary.store(on ? 1 : 0);
  return TSIM_OK;
}

extern "C" int tsim_debug_set_wait_limit(int64_t attempts) {
  return tsim::set_wait_limit((long long)attempts);
}

extern "C" int tsim_probe_fp32_tflops(tsim_ctx* ctx, double* tflops) {
  TSIM_CHECK_ARG(ctx && tflops, "NULL argument");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  const int blocks = ctx->num_sms * 8, threads = 256, iters = 4096;
  float* out = reinterpret_cast<float*>(ctx->dcounters) + 8;
  fp32_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(out, 64, 1.0000001f, 1e-7f);  // warm
  TSIM_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  fp32_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters, 1.0000001f, 1e-7f);
  TSIM_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  TSIM_CUDA(cudaEventSynchronize(ctx->ev1));
  float ms = 0.0f;
  TSIM_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  launched(ctx, 2);
  const double flops = 2.0 * kChains * iters * (double)blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return TSIM_OK;
}

extern "C" {

const char* tsim_status_string(int s) {
  switch (s) {
    case TSIM_OK: return "ok";
    case TSIM_ERR_INVALID_ARG: return "invalid argument";
    case TSIM_ERR_CUDA: return "CUDA error";
    case TSIM_ERR_OUT_OF_MEMORY: return "out of device memory";
    case TSIM_ERR_TIMEOUT: return "bounded wait timed out";
    case TSIM_ERR_UNSUPPORTED: return "unsupported";
    case TSIM_ERR_BUDGET: return "over admission budget";
    case TSIM_PENDING: return "pending";
    case TSIM_ERR_BUSY: return "admission queue full";
  }
  return "unknown status";
}

const char* tsim_last_error(void) { return g_last_error.c_str(); }

int tsim_version(void) { return 10000; }

int tsim_ctx_create(int device, void* stream, tsim_ctx** out) {
  TSIM_CHECK_ARG(out != nullptr, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  TSIM_CUDA(cudaGetDeviceCount(&ndev));
  TSIM_CHECK_ARG(device >= 0 && device < ndev, "no such CUDA device");
  TSIM_CUDA(cudaSetDevice(device));
  tsim_ctx* c = new tsim_ctx;
  c->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaGetDeviceProperties", __FILE__, __LINE__);
  }
  c->num_sms = prop.multiProcessorCount;
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    c->owns_stream = true;
  }
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  e = dev_malloc(reinterpret_cast<void**>(&c->dcounters), 64 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(c->dcounters, 0, 64 * sizeof(unsigned long long));
  if (e == cudaSuccess) c->status = reinterpret_cast<unsigned*>(c->dcounters + kStatusSlot);
  if (e != cudaSuccess) {
    if (c->owns_stream) cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(e, "tsim_ctx_create counters", __FILE__, __LINE__);
  }
  *out = c;
  return TSIM_OK;
}

static void db_free(tsim_db* db);

int tsim_ctx_destroy(tsim_ctx* c) {
  if (!c) return TSIM_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& g : c->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  for (tsim_ctx* s : c->subs) tsim_ctx_destroy(s);
  c->subs.clear();
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  for (auto ev : c->join_ev) cudaEventDestroy(ev);
  c->join_ev.clear();
  for (tsim_db* db : c->dbs) {  // detach: free device memory, keep the handle
    db_free(db);
    db->ctx = nullptr;
  }
  c->dbs.clear();
  if (c->arena && !c->arena_external) cudaFree(c->arena);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->hstage) cudaFree(c->hstage);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (auto& ev : c->stage_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->dcounters) cudaFree(c->dcounters);
  if (c->owns_stream) cudaStreamDestroy(c->stream);
  delete c;
  return TSIM_OK;
}

int tsim_ctx_set_stream(tsim_ctx* c, void* stream) {
  TSIM_CHECK_ARG(c != nullptr, "ctx is NULL");
  TSIM_CUDA(cudaStreamSynchronize(c->stream));
  if (c->owns_stream) cudaStreamDestroy(c->stream);
  c->owns_stream = false;
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    TSIM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->owns_stream = true;
  }
  return TSIM_OK;
}

int tsim_ctx_synchronize(tsim_ctx* c) {
  TSIM_CHECK_ARG(c != nullptr, "ctx is NULL");
  TSIM_CUDA(cudaStreamSynchronize(c->stream));
  return TSIM_OK;
}

int64_t tsim_ctx_scratch_bytes(const tsim_ctx* c) { return c ? (int64_t)c->arena_cap : 0; }

static int db_alloc(tsim_db* db) {
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&db->segbox), sizeof(float4) * kSegs * std::max(db->count, 1)));
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&db->segsum), sizeof(float2) * kSegs * std::max(db->count, 1)));
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&db->box), sizeof(float4) * std::max(db->count, 1)));
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&db->ends), sizeof(float4) * std::max(db->count, 1)));
  TSIM_CUDA(dev_malloc(reinterpret_cast<void**>(&db->len), sizeof(int) * std::max(db->count, 1)));
  return TSIM_OK;
}

static void db_free(tsim_db* db) {
  if (db->owns) {
    cudaFree(db->pts);
    cudaFree(db->off);
  }
  cudaFree(db->box);
  cudaFree(db->ends);
  cudaFree(db->len);
  cudaFree(db->segbox);
  cudaFree(db->segsum);
  db->segbox = nullptr;
  db->segsum = nullptr;
  db->pts = nullptr;
  db->off = nullptr;
  db->box = db->ends = nullptr;
  db->len = nullptr;
}

int tsim_db_create(tsim_ctx* ctx, const tsim_point* h_pts, const int64_t* h_off, int count,
                   tsim_db** out) {
  TSIM_CHECK_ARG(ctx && out && h_off && count >= 0, "bad arguments");
  *out = nullptr;
  TSIM_CHECK_ARG(h_off[0] == 0, "offsets must start at 0");
  int max_len = 0;
  for (int t = 0; t < count; ++t) {
    TSIM_CHECK_ARG(h_off[t + 1] > h_off[t], "trajectories must be non-empty (offsets increasing)");
    TSIM_CHECK_ARG(h_off[t + 1] - h_off[t] <= INT32_MAX, "trajectory longer than 2^31 - 1 points");
    max_len = std::max<int64_t>(max_len, h_off[t + 1] - h_off[t]);
  }
  TSIM_CHECK_ARG(h_pts != nullptr || count == 0, "h_pts is NULL");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  tsim_db* db = new tsim_db;
  db->ctx = ctx;
  db->count = count;
  db->total = h_off[count];
  db->max_len = max_len;
  db->owns = true;
  db->h_off.assign(h_off, h_off + count + 1);
  int s = TSIM_OK;
  cudaError_t e = dev_malloc(reinterpret_cast<void**>(&db->pts),
                             sizeof(float2) * std::max<int64_t>(db->total, 1));
  if (e == cudaSuccess)
    e = dev_malloc(reinterpret_cast<void**>(&db->off), sizeof(int64_t) * (count + 1));
  if (e == cudaSuccess && db->total > 0)
    e = cudaMemcpyAsync(db->pts, h_pts, sizeof(float2) * db->total, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(db->off, h_off, sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e != cudaSuccess) s = cuda_fail(e, "tsim_db_create upload", __FILE__, __LINE__);
  if (s == TSIM_OK) s = db_alloc(db);
  if (s == TSIM_OK) s = db_summarize(db);
  if (s == TSIM_OK) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = cuda_fail(e, "tsim_db_create sync", __FILE__, __LINE__);
  }
  if (s != TSIM_OK) {
    db_free(db);
    delete db;
    return s;
  }
  ctx->dbs.push_back(db);
  *out = db;
  return TSIM_OK;
}

int tsim_db_wrap_device(tsim_ctx* ctx, const tsim_point* d_pts, const int64_t* d_off, int count,
                        int max_len, tsim_db** out) {
  TSIM_CHECK_ARG(ctx && out && d_off && count >= 0, "bad arguments");
  *out = nullptr;
  TSIM_CUDA(cudaSetDevice(ctx->device));
  tsim_db* db = new tsim_db;
  db->ctx = ctx;
  db->count = count;
  db->owns = false;
  db->pts = (float2*)d_pts;
  db->off = (int64_t*)d_off;
  db->h_off.resize(count + 1);
  cudaError_t e = cudaMemcpyAsync(db->h_off.data(), d_off, sizeof(int64_t) * (count + 1),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    delete db;
    return cuda_fail(e, "tsim_db_wrap_device offsets", __FILE__, __LINE__);
  }
  db->total = db->h_off[count];
  int ml = 0;
  for (int t = 0; t < count; ++t) {
    if (db->h_off[t + 1] <= db->h_off[t] || db->h_off[0] != 0 ||
        db->h_off[t + 1] - db->h_off[t] > INT32_MAX) {
      delete db;
      return fail(TSIM_ERR_INVALID_ARG, "tsim_db_wrap_device: offsets must start at 0 and increase by at most 2^31 - 1");
    }
    ml = std::max<int64_t>(ml, db->h_off[t + 1] - db->h_off[t]);
  }
  (void)max_len;  // the offsets, read here anyway, give the exact value
  db->max_len = ml;
  int s = db_alloc(db);
  if (s == TSIM_OK) s = db_summarize(db);
  if (s == TSIM_OK) {
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = cuda_fail(e, "tsim_db_wrap_device sync", __FILE__, __LINE__);
  }
  if (s != TSIM_OK) {
    db_free(db);
    delete db;
    return s;
  }
  ctx->dbs.push_back(db);
  *out = db;
  return TSIM_OK;
}

int tsim_db_destroy(tsim_db* db) {
  if (!db) return TSIM_OK;
  if (db->ctx) {  // still attached: release its memory and unregister it
    cudaSetDevice(db->ctx->device);
    cudaStreamSynchronize(db->ctx->stream);
    for (auto& g : db->ctx->graphs)  // captured graphs may reference this database
      if (g.exec) cudaGraphExecDestroy(g.exec);
    db->ctx->graphs.clear();
    db_free(db);
    auto& v = db->ctx->dbs;
    v.erase(std::remove(v.begin(), v.end(), db), v.end());
  }
  delete db;
  return TSIM_OK;
}

int tsim_db_count(const tsim_db* db) { return db ? db->count : 0; }

int64_t tsim_db_device_bytes(const tsim_db* db) {
  if (!db) return 0;
  return (db->owns ? (int64_t)sizeof(float2) * db->total + 8 * (db->count + 1) : 0) +
         (int64_t)db->count * (16 + 16 + 4 + (16 + 8) * kSegs);
}

}  // extern "C"
