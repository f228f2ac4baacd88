// tune.cu -- the autotuner: launch choices of the exact kNN path picked by
// measurement on this GPU, per request shape class.
//
// Two choices are tuned: the first rows per lane-group R of the anti-diagonal
// DP's survivor passes (1 .. 16; 0 runs every pair on the round-striped kernel) and the number
// of query chunks a request runs concurrently on child streams (1, 2, 4, 8).
// tsim_autotune times every admissible pair of choices on the caller's own
// request (device pointers, CUDA events on the context stream, the median of
// `reps` runs after one warm-up run) and records the fastest in the
// context's table under the request's shape class (measure, cost, band,
// window, k and the log2 buckets of the longest query, the longest
// candidate, the database size and the query count).  Later requests of
// that class use the recorded choices; the table can be saved to and loaded
// from a text file (one line per class, tagged with the device name).
// Results do not depend on the choices: every configuration computes the
// same cells with the same operations.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tsim_internal.cuh"

namespace tsim {
namespace {

std::string device_name(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string n = prop.name;
  for (char& c : n)
    if (c == ' ' || c == '\t' || c == '\n') c = '_';
  return n;
}

// smallest R whose anti-diagonal validity condition holds for the longest
// query against the longest candidate (16 when none does)
int min_rdiag(const tsim_params* p, int max_qlen, const tsim_db* db) {
  const int n = max_qlen, m = db->max_len;
  const int wd = p->measure == TSIM_LCSS ? p->delta
                                         : (p->measure == TSIM_DTW ? band_w(n, m, p->band_pct) : -1);
  for (int R : {1, 2, 4, 8, 16})
    if (diag_ok(p->measure == TSIM_LCSS, n, m, wd, R)) return R;
  return 16;
}

}  // namespace
}  // namespace tsim

using namespace tsim;

extern "C" int tsim_autotune(tsim_ctx* ctx, const tsim_params* p, const tsim_point* d_qpts,
                             const int64_t* d_qoff, int nq, int max_qlen, tsim_db* db, int reps,
                             tsim_tune_result* out) {
  TSIM_CHECK_ARG(ctx && p && db && d_qpts && d_qoff, "NULL argument");
  TSIM_CHECK_ARG(db->ctx == ctx, "database belongs to another (or a destroyed) context");
  TSIM_CHECK_ARG(nq >= 1 && max_qlen >= 1 && p->k >= 1 && p->k <= 64, "bad sizes");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  reps = std::max(1, std::min(reps, 50));
  tsim_params q = *p;
  q.flags |= TSIM_FLAG_NO_GRAPH;
  const std::vector<int> key = tune_key(p, nq, max_qlen, db);
  // candidates
  std::vector<int> rs{0};
  const bool dp = p->measure == TSIM_DTW || p->measure == TSIM_LCSS || p->measure == TSIM_FRECHET;
  if (dp) {
    // from half the longest pair's R (narrow-band pairs at fewer rows per
    // lane in a first pass, the rest in the next) to four times it; with
    // full rows (no band, no window) every R from 1: a pair needs as many
    // rows per lane-group as its candidate is long, so a chain from R = 1
    // runs each pair at the fewest its length admits
    const int r0 = min_rdiag(p, max_qlen, db);
    const bool full_rows = p->measure == TSIM_FRECHET ||
                           (p->measure == TSIM_DTW && p->band_pct < 0) ||
                           (p->measure == TSIM_LCSS && p->delta < 0);
    for (int R : {1, 2, 4, 8, 16})
      if (full_rows || (2 * R >= r0 && R <= 4 * r0)) rs.push_back(R);
  }
  std::vector<int> ss;
  for (int s : {1, 2, 4, 8})
    if (s == 1 || s <= nq / 8) ss.push_back(s);
  // scratch outputs and events
  int* ids = nullptr;
  float* dd = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = TSIM_OK;
  cudaError_t ce = dev_malloc(reinterpret_cast<void**>(&ids), sizeof(int) * (size_t)nq * p->k);
  if (ce == cudaSuccess) ce = dev_malloc(reinterpret_cast<void**>(&dd), sizeof(float) * (size_t)nq * p->k);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) st = cuda_fail(ce, "tsim_autotune setup", __FILE__, __LINE__);
  const bool had = ctx->tuning.count(key) > 0;
  const tsim_ctx::TuneVal saved = had ? ctx->tuning[key] : tsim_ctx::TuneVal{};
  auto time_config = [&](bool use_table, int R, int S, double& med) -> int {
    if (use_table) {
      tsim_ctx::TuneVal v;
      v.rdiag = R;
      v.streams = S;
      ctx->tuning[key] = v;
    } else {
      ctx->tuning.erase(key);
    }
    std::vector<double> t;
    for (int i = 0; i <= reps; ++i) {
      TSIM_CUDA(cudaEventRecord(e0, ctx->stream));
      TSIM_TRY(knn_request(ctx, &q, d_qpts, d_qoff, nq, max_qlen, db, ids, dd, nullptr, nullptr));
      TSIM_CUDA(cudaEventRecord(e1, ctx->stream));
      TSIM_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      TSIM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (i > 0) t.push_back(ms);  // the first run warms up (and sizes the scratch)
    }
    std::sort(t.begin(), t.end());
    med = t[t.size() / 2];
    return TSIM_OK;
  };
  double def_ms = 0.0, best_ms = 1e300;
  int best_r = -1, best_s = ctx->concurrency, tried = 0;
  if (st == TSIM_OK) st = time_config(false, -1, 0, def_ms);
  for (int R : rs) {
    for (int S : ss) {
      if (st != TSIM_OK) break;
      double ms = 0.0;
      st = time_config(true, R, S, ms);
      ++tried;
      if (st == TSIM_OK && ms < best_ms) {
        best_ms = ms;
        best_r = R;
        best_s = S;
      }
    }
  }
  if (st == TSIM_OK) {
    tsim_ctx::TuneVal v;
    v.rdiag = best_r;
    v.streams = best_s;
    v.ms = best_ms;
    ctx->tuning[key] = v;
  } else if (had) {
    ctx->tuning[key] = saved;
  } else {
    ctx->tuning.erase(key);
  }
  if (ids) cudaFree(ids);
  if (dd) cudaFree(dd);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st != TSIM_OK) return st;
  if (out) {
    out->rdiag = best_r;
    out->streams = best_s;
    out->best_ms = best_ms;
    out->default_ms = def_ms;
    out->tried = tried;
  }
  return TSIM_OK;
}

extern "C" int tsim_tuning_count(const tsim_ctx* ctx) { return ctx ? (int)ctx->tuning.size() : 0; }

extern "C" int tsim_tuning_clear(tsim_ctx* ctx) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  ctx->tuning.clear();
  return TSIM_OK;
}

extern "C" int tsim_tuning_save(tsim_ctx* ctx, const char* path) {
  TSIM_CHECK_ARG(ctx && path, "NULL argument");
  FILE* f = fopen(path, "w");
  if (!f) return fail(TSIM_ERR_INVALID_ARG, std::string("cannot write ") + path);
  fprintf(f, "# tsim tuning v1 %s\n", device_name(ctx->device).c_str());
  fprintf(f, "# measure cost band delta k log2_qlen log2_clen log2_count log2_nq rdiag streams ms\n");
  for (const auto& kv : ctx->tuning) {
    for (int v : kv.first) fprintf(f, "%d ", v);
    fprintf(f, "%d %d %.6f\n", kv.second.rdiag, kv.second.streams, kv.second.ms);
  }
  const bool ok = fclose(f) == 0;
  return ok ? TSIM_OK : fail(TSIM_ERR_INVALID_ARG, std::string("cannot write ") + path);
}

extern "C" int tsim_tuning_load(tsim_ctx* ctx, const char* path) {
  TSIM_CHECK_ARG(ctx && path, "NULL argument");
  FILE* f = fopen(path, "r");
  if (!f) return fail(TSIM_ERR_INVALID_ARG, std::string("cannot read ") + path);
  char line[512];
  const std::string dev = device_name(ctx->device);
  bool header = false;
  std::vector<std::pair<std::vector<int>, tsim_ctx::TuneVal>> rows;
  int st = TSIM_OK;
  while (fgets(line, sizeof(line), f)) {
    if (line[0] == '#') {
      char name[256] = {0};
      if (sscanf(line, "# tsim tuning v1 %255s", name) == 1) {
        header = true;
        if (dev != name) {
          st = fail(TSIM_ERR_UNSUPPORTED, std::string("tuning file is for ") + name + ", not " + dev);
          break;
        }
      }
      continue;
    }
    std::vector<int> key(9);
    tsim_ctx::TuneVal v;
    const int got = sscanf(line, "%d %d %d %d %d %d %d %d %d %d %d %lf", &key[0], &key[1], &key[2],
                           &key[3], &key[4], &key[5], &key[6], &key[7], &key[8], &v.rdiag,
                           &v.streams, &v.ms);
    if (got == EOF || (got == 0 && strspn(line, " \t\r\n") == strlen(line))) continue;
    if (got != 12 || v.rdiag < -1 || v.rdiag > 16 || v.streams < 1 || v.streams > 64) {
      st = fail(TSIM_ERR_INVALID_ARG, std::string("malformed tuning line: ") + line);
      break;
    }
    rows.emplace_back(key, v);
  }
  fclose(f);
  if (st == TSIM_OK && !header) st = fail(TSIM_ERR_INVALID_ARG, "not a tuning file (no header)");
  if (st != TSIM_OK) return st;
  for (auto& r : rows) ctx->tuning[r.first] = r.second;
  return TSIM_OK;
}
