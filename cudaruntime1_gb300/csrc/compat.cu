// compat.cu -- the reference's GPU entry points, same names and signatures
// (CudaRuntime1/dtw.cuh:6, lcss.cuh:6-7, frechet.cuh:6, hausdorff.cuh:11-19,
// euclidean.cuh:10-13), implemented over the C ABI.
//
// Contract kept from the reference: host pointers in and out, one float per
// query, synchronous, `gpu_time` in milliseconds (total wall time for the
// pipelines, kernel time for launch_hausdorff_rtree_gpu and
// execute_rtree_csr_kernel_on_gpu, as the reference reports them).  Error
// behaviour: the reference's CHECK prints and exits (common.cuh:14-22); so do
// these, unless TSIM_COMPAT_NO_EXIT is set in the environment, in which case
// they print, fill the results with NaN and return.
//
// Device buffers are cached between calls instead of cudaMalloc/cudaFree per
// call (dtw.cu:131-134, 222-223).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "../../include/compat/dtw.cuh"
#include "../../include/compat/euclidean.cuh"
#include "../../include/compat/frechet.cuh"
#include "../../include/compat/hausdorff.cuh"
#include "../../include/compat/lcss.cuh"
#include "tsim_internal.cuh"

static_assert(sizeof(Point) == sizeof(tsim_point), "Point layout");

namespace {

std::mutex g_mu;
tsim_ctx* g_ctx = nullptr;
int g_dev = -1;

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};
DevBuf g_buf[6];

bool ensure(DevBuf& b, size_t bytes) {
  if (bytes <= b.cap) return true;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t cap = bytes + bytes / 8 + 256;
  if (tsim::dev_malloc(reinterpret_cast<void**>(&b.p), cap) != cudaSuccess) {
    tsim::set_error("cudaMalloc of compat buffer failed");
    return false;
  }
  b.cap = cap;
  return true;
}

tsim_ctx* ctx() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (g_ctx && g_dev != dev) {  // the cached buffers live on the previous device
    cudaSetDevice(g_dev);
    tsim_ctx_destroy(g_ctx);
    g_ctx = nullptr;
    for (auto& b : g_buf) {
      if (b.p) cudaFree(b.p);
      b = DevBuf{};
    }
    cudaSetDevice(dev);
  }
  if (!g_ctx) {
    if (tsim_ctx_create(dev, nullptr, &g_ctx) != TSIM_OK) return nullptr;
    g_dev = dev;
  }
  return g_ctx;
}

void fail_call(const char* where, float* out, int count) {
  fprintf(stderr, "Error: %s: %s\n", where, tsim_last_error());
  if (!getenv("TSIM_COMPAT_NO_EXIT")) exit(1);
  for (int i = 0; i < count; ++i) out[i] = NAN;
}

double ms_since(std::chrono::high_resolution_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0)
      .count();
}

#define COMPAT_TRY(expr)       \
  do {                         \
    if (!(expr)) return false; \
  } while (0)

bool h2d(tsim_ctx* c, DevBuf& b, const void* h, size_t bytes) {
  COMPAT_TRY(ensure(b, bytes));
  if (bytes == 0) return true;
  cudaError_t e = cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) tsim::set_error(cudaGetErrorString(e));
  return e == cudaSuccess;
}

bool d2h_sync(tsim_ctx* c, void* h, const void* d, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) tsim::set_error(cudaGetErrorString(e));
  return e == cudaSuccess;
}

bool ref_batch_host(int measure, const Point* t1, const Point* t2, float* out, int num_t, int n,
                    int m, float eps) {
  tsim_ctx* c = ctx();
  COMPAT_TRY(c);
  COMPAT_TRY(h2d(c, g_buf[0], t1, sizeof(Point) * (size_t)num_t * n));
  COMPAT_TRY(h2d(c, g_buf[1], t2, sizeof(Point) * (size_t)num_t * m));
  COMPAT_TRY(ensure(g_buf[2], sizeof(float) * num_t));
  COMPAT_TRY(tsim_ref_batch(c, measure, (const tsim_point*)g_buf[0].p, (const tsim_point*)g_buf[1].p,
                            num_t, n, m, eps, (float*)g_buf[2].p) == TSIM_OK);
  return d2h_sync(c, out, g_buf[2].p, sizeof(float) * num_t);
}

bool hausdorff_host(const Point* t1, int num_t1, int n, const Point* t2, int num_t2, int m,
                    const int* h_cand, int top_k, float* out, float* kernel_ms) {
  tsim_ctx* c = ctx();
  COMPAT_TRY(c);
  COMPAT_TRY(h2d(c, g_buf[0], t1, sizeof(Point) * (size_t)num_t1 * n));
  COMPAT_TRY(h2d(c, g_buf[1], t2, sizeof(Point) * (size_t)num_t2 * m));
  COMPAT_TRY(ensure(g_buf[2], sizeof(float) * num_t1));
  COMPAT_TRY(ensure(g_buf[3], sizeof(int) * (size_t)num_t1 * top_k));
  if (h_cand) {
    COMPAT_TRY(h2d(c, g_buf[3], h_cand, sizeof(int) * (size_t)num_t1 * top_k));
  } else {
    COMPAT_TRY(tsim_mbr_knn(c, (const tsim_point*)g_buf[0].p, num_t1, n,
                            (const tsim_point*)g_buf[1].p, num_t2, m, top_k,
                            (int*)g_buf[3].p) == TSIM_OK);
  }
  cudaEventRecord(c->ev0, c->stream);
  COMPAT_TRY(tsim_hausdorff_cands(c, (const tsim_point*)g_buf[0].p, num_t1, n,
                                  (const tsim_point*)g_buf[1].p, num_t2, m, (const int*)g_buf[3].p,
                                  top_k, (float*)g_buf[2].p) == TSIM_OK);
  cudaEventRecord(c->ev1, c->stream);
  COMPAT_TRY(d2h_sync(c, out, g_buf[2].p, sizeof(float) * num_t1));
  if (kernel_ms) cudaEventElapsedTime(kernel_ms, c->ev0, c->ev1);
  return true;
}

bool euclid_host(const Point* t1, const Point* t2, const int* h_cand, const int* h_off, int num_t,
                 int n, int total, float* out, float* kernel_ms) {
  tsim_ctx* c = ctx();
  COMPAT_TRY(c);
  COMPAT_TRY(h2d(c, g_buf[0], t1, sizeof(Point) * (size_t)num_t * n));
  COMPAT_TRY(h2d(c, g_buf[1], t2, sizeof(Point) * (size_t)num_t * n));
  COMPAT_TRY(ensure(g_buf[2], sizeof(float) * num_t));
  int k = std::min(50, num_t);
  if (h_cand) {
    COMPAT_TRY(h2d(c, g_buf[3], h_cand, sizeof(int) * (size_t)std::max(total, 1)));
    COMPAT_TRY(h2d(c, g_buf[4], h_off, sizeof(int) * (size_t)(num_t + 1)));
  } else {
    // the R-tree's k = min(50, num_t) nearest boxes per query
    // (euclidean_rtree.cpp:57-68), as a fixed-stride CSR
    total = num_t * k;
    COMPAT_TRY(ensure(g_buf[3], sizeof(int) * (size_t)total));
    std::vector<int> off(num_t + 1);
    for (int i = 0; i <= num_t; ++i) off[i] = i * k;
    COMPAT_TRY(h2d(c, g_buf[4], off.data(), sizeof(int) * (num_t + 1)));
    COMPAT_TRY(tsim_mbr_knn(c, (const tsim_point*)g_buf[0].p, num_t, n,
                            (const tsim_point*)g_buf[1].p, num_t, n, k, (int*)g_buf[3].p) == TSIM_OK);
    // the host vector above must outlive the async copy
    COMPAT_TRY(cudaStreamSynchronize(c->stream) == cudaSuccess);
  }
  cudaEventRecord(c->ev0, c->stream);
  COMPAT_TRY(tsim_euclid_cands(c, (const tsim_point*)g_buf[0].p, (const tsim_point*)g_buf[1].p,
                               (const int*)g_buf[3].p, (const int*)g_buf[4].p, num_t, n, total,
                               (float*)g_buf[2].p) == TSIM_OK);
  cudaEventRecord(c->ev1, c->stream);
  COMPAT_TRY(d2h_sync(c, out, g_buf[2].p, sizeof(float) * num_t));
  if (kernel_ms) cudaEventElapsedTime(kernel_ms, c->ev0, c->ev1);
  return true;
}

}  // namespace

#pragma GCC visibility push(default)

void launch_dtw_batch_gpu_knn(const Point* h_t1, const Point* h_t2, float* h_results, int num_t,
                              int n, int m, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::high_resolution_clock::now();
  if (!ref_batch_host(TSIM_DTW, h_t1, h_t2, h_results, num_t, n, m, 0.0f))
    fail_call("launch_dtw_batch_gpu_knn", h_results, num_t);
  gpu_time = (float)ms_since(t0);
}

void launch_lcss_batch_gpu_wavefront_knn(const Point* h_t1, const Point* h_t2, float* h_results,
                                         int num_t, int n, int m, float epsilon, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::high_resolution_clock::now();
  if (!ref_batch_host(TSIM_LCSS, h_t1, h_t2, h_results, num_t, n, m, epsilon))
    fail_call("launch_lcss_batch_gpu_wavefront_knn", h_results, num_t);
  gpu_time = (float)ms_since(t0);
}

void launch_frechet_batch_gpu_wavefront(const Point* h_t1, const Point* h_t2, float* h_results,
                                        int num_t, int n, int m, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::high_resolution_clock::now();
  if (!ref_batch_host(TSIM_FRECHET, h_t1, h_t2, h_results, num_t, n, m, 0.0f))
    fail_call("launch_frechet_batch_gpu_wavefront", h_results, num_t);
  gpu_time = (float)ms_since(t0);
}

float run_hausdorff_rtree_gpu_pipeline(const Point* h_t1, int num_t1, int n, const Point* h_t2,
                                       int num_t2, int m, float* h_results, int top_k) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::high_resolution_clock::now();
  if (!hausdorff_host(h_t1, num_t1, n, h_t2, num_t2, m, nullptr, top_k, h_results, nullptr))
    fail_call("run_hausdorff_rtree_gpu_pipeline", h_results, num_t1);
  return (float)ms_since(t0);
}

void launch_hausdorff_rtree_gpu(const Point* h_t1, int num_t1, int n, const Point* h_t2,
                                int num_t2, int m, const int* h_candidate_indices, int top_k,
                                float* h_results, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  float ms = 0.0f;
  if (!h_candidate_indices) {
    tsim::set_error("h_candidate_indices is NULL");
    fail_call("launch_hausdorff_rtree_gpu", h_results, num_t1);
  } else if (!hausdorff_host(h_t1, num_t1, n, h_t2, num_t2, m, h_candidate_indices, top_k,
                             h_results, &ms)) {
    fail_call("launch_hausdorff_rtree_gpu", h_results, num_t1);
  }
  gpu_time = ms;
}

void launch_euclidean_batch_gpu_rtree_exact(const Point* h_t1, const Point* h_t2,
                                            float* h_results, int num_t, int n, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::high_resolution_clock::now();
  if (!euclid_host(h_t1, h_t2, nullptr, nullptr, num_t, n, 0, h_results, nullptr))
    fail_call("launch_euclidean_batch_gpu_rtree_exact", h_results, num_t);
  gpu_time = (float)ms_since(t0);
}

void execute_rtree_csr_kernel_on_gpu(const Point* h_t1, const Point* h_t2, const int* h_candidates,
                                     const int* h_offsets, float* h_results, int num_t, int n,
                                     int total_candidates, float& gpu_time) {
  std::lock_guard<std::mutex> lk(g_mu);
  float ms = 0.0f;
  if (!h_offsets || (total_candidates > 0 && !h_candidates)) {
    tsim::set_error("NULL candidate arrays");
    fail_call("execute_rtree_csr_kernel_on_gpu", h_results, num_t);
  } else if (!euclid_host(h_t1, h_t2, h_candidates, h_offsets, num_t, n, total_candidates,
                          h_results, &ms)) {
    fail_call("execute_rtree_csr_kernel_on_gpu", h_results, num_t);
  }
  gpu_time = ms;
}

#pragma GCC visibility pop
