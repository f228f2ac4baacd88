// pairwise_knn.cu -- refine kernels of the exact kNN path for symmetric
// Hausdorff and lock-step Euclidean: one warp per (query, candidate) pair.
//
// Hausdorff (FP32): lane l holds query points l, l+32, ... in registers and
// streams the candidate's points (every lane reads the same point: one
// broadcast transaction), keeping each point's minimum squared distance; the
// warp maximum is h(Q,C).  The reverse direction swaps the roles.  A pair
// whose running maximum already exceeds the query's threshold is abandoned.
// Reference kernel replaced: hausdorff_tiled_rtree_kernel
// (CudaRuntime1/hausdorff.cu:84-122), one CTA per query over 256-point tiles.
//
// Euclidean: lane-strided sum of squared point differences, compensated
// FP32 (TwoSum) for candidates of up to 1024 points, FP64 beyond (the error
// of an uncompensated FP32 sum grows with length).  Reference kernel
// replaced: euclidean_rtree_csr_kernel_global (CudaRuntime1/euclidean.cu:17-73).
//
// FP64 kernels compute the oracle's arithmetic (oracle/oracle.c
// orc_hausdorff64, orc_euclid64) for the pairs the FP32 values cannot order.
#include "dfloat.cuh"
#include "tsim_internal.cuh"

namespace tsim {
namespace {

constexpr int kPwThreads = 128;
constexpr int kMaxRegPts = 8;  // query points per lane kept in registers

__device__ __forceinline__ float d2f(float ax, float ay, float bx, float by) {
  const float dx = ax - bx, dy = ay - by;
  return fmaf(dy, dy, dx * dx);
}

// max over S of min over T of |s - t|^2 (FP32); stops above `stop`.
// *pairs (lane 0's copy) grows by the point pairs compared.
__device__ float warp_directed(const float2* S, int ns, const float2* T, int nt, float run,
                               float stop, long long* pairs) {
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < ns; base += 32 * kMaxRegPts) {
    *pairs += (long long)min(32 * kMaxRegPts, ns - base) * nt;
    float sx[kMaxRegPts], sy[kMaxRegPts], mn[kMaxRegPts];
#pragma unroll
    for (int u = 0; u < kMaxRegPts; ++u) {
      const int i = base + u * 32 + lane;
      const float2 p = i < ns ? S[i] : S[0];
      sx[u] = p.x;
      sy[u] = p.y;
      mn[u] = TSIM_INF;
    }
    const int nu = min(kMaxRegPts, (ns - base + 31) / 32);
    for (int j = 0; j < nt; ++j) {
      const float2 t = T[j];
#pragma unroll
      for (int u = 0; u < kMaxRegPts; ++u)
        if (u < nu) mn[u] = fminf(mn[u], d2f(sx[u], sy[u], t.x, t.y));
    }
    float loc = 0.0f;
#pragma unroll
    for (int u = 0; u < kMaxRegPts; ++u)
      if (base + u * 32 + lane < ns) loc = fmaxf(loc, mn[u]);
    for (int o = 16; o; o >>= 1) loc = fmaxf(loc, __shfl_xor_sync(0xffffffffu, loc, o));
    run = fmaxf(run, loc);
    if (run > stop) return run;
  }
  return run;
}

__global__ void __launch_bounds__(kPwThreads) hausdorff_refine_kernel(PwArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;
  for (int w = gw; w < npairs; w += nw) {
    const int pid = a.order ? a.order[w] : w;
    const int2 pr = a.pairs[pid];
    if (pr.y < 0) continue;
    const int64_t qo = a.qoff[pr.x], co = a.coff[pr.y];
    const int n = (int)(a.qoff[pr.x + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    float v = TSIM_INF;
    long long pairs = 0;
    if (n > 0 && m > 0) {
      const float stop = a.thr ? a.thr[pr.x] : TSIM_INF;
      v = warp_directed(a.qpts + qo, n, a.cpts + co, m, 0.0f, stop, &pairs);
      if (v <= stop) v = warp_directed(a.cpts + co, m, a.qpts + qo, n, v, stop, &pairs);
      if (v > stop) v = TSIM_INF;  // abandoned: cannot be among the k best
    }
    if (lane == 0) {
      a.out[pid] = v;
      if (a.cells && pairs) atomicAdd(a.cells, (unsigned long long)pairs);
    }
  }
}

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float t) {
  float ns, e;
  two_sum_f(s, t, ns, e);
  s = ns;
  c += e;
}

// lock-step sum over the candidate's m points against the query's first m
// (+inf when the query is shorter)
__global__ void __launch_bounds__(kPwThreads) euclid_refine_kernel(PwArgs a) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int npairs = a.npairs_dev ? min(*a.npairs_dev, a.npairs) : a.npairs;
  for (int w = gw; w < npairs; w += nw) {
    const int pid = a.order ? a.order[w] : w;
    const int2 pr = a.pairs[pid];
    if (pr.y < 0) continue;
    const int64_t qo = a.qoff[pr.x], co = a.coff[pr.y];
    const int n = (int)(a.qoff[pr.x + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    const float2* A = a.qpts + qo;
    const float2* B = a.cpts + co;
    float v = TSIM_INF;
    if (n >= m && m > 0) {
      if (m <= 1024) {
        float s = 0.0f, c = 0.0f;
        for (int i = lane; i < m; i += 32) {
          const float2 p = A[i], r = B[i];
          two_sum_acc(s, c, d2f(p.x, p.y, r.x, r.y));
        }
        for (int o = 16; o; o >>= 1) {
          const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
          const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
          float ns, e;
          two_sum_f(s, s2, ns, e);
          s = ns;
          c = c + c2 + e;
        }
        v = s + c;
      } else {
        double s = 0.0;
        for (int i = lane; i < m; i += 32) {
          const float2 p = A[i], r = B[i];
          const double dx = (double)p.x - (double)r.x, dy = (double)p.y - (double)r.y;
          s += dx * dx + dy * dy;
        }
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        v = __double2float_rn(s);
      }
      const float stop = a.thr ? a.thr[pr.x] : TSIM_INF;
      if (v > stop) v = TSIM_INF;
    }
    if (lane == 0) {
      a.out[pid] = v;
      if (a.cells && n >= m && m > 0) atomicAdd(a.cells, (unsigned long long)m);
    }
  }
}

// ---- FP64 (the oracle's arithmetic) -----------------------------------------
__device__ __forceinline__ double d2_64f(float ax, float ay, float bx, float by) {
  const double dx = (double)ax - (double)bx, dy = (double)ay - (double)by;
  return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

__device__ double warp_directed64(const float2* S, int ns, const float2* T, int nt) {
  const int lane = threadIdx.x & 31;
  double run = 0.0;
  for (int i0 = 0; i0 < ns; i0 += 32) {
    const int i = i0 + lane;
    double mn = __longlong_as_double(0x7ff0000000000000ll);
    if (i < ns) {
      const float2 p = S[i];
      for (int j = 0; j < nt; ++j) {
        const float2 t = T[j];
        const double d = d2_64f(p.x, p.y, t.x, t.y);
        mn = d < mn ? d : mn;
      }
    } else {
      mn = 0.0;
    }
    for (int o = 16; o; o >>= 1) {
      const double x = __shfl_xor_sync(0xffffffffu, mn, o);
      mn = x > mn ? x : mn;
    }
    run = mn > run ? mn : run;
  }
  return run;
}

__global__ void __launch_bounds__(kPwThreads) pairwise64_kernel(PwArgs a, int euclid) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int w = gw; w < a.npairs; w += nw) {
    const int2 pr = a.pairs[w];
    if (pr.y < 0) continue;
    const int64_t qo = a.qoff[pr.x], co = a.coff[pr.y];
    const int n = (int)(a.qoff[pr.x + 1] - qo), m = (int)(a.coff[pr.y + 1] - co);
    const float2* A = a.qpts + qo;
    const float2* B = a.cpts + co;
    double v = __longlong_as_double(0x7ff0000000000000ll);
    if (euclid) {
      if (n >= m && m > 0 && lane == 0) {  // left to right, as the oracle sums
        double s = 0.0;
        for (int i = 0; i < m; ++i) s = __dadd_rn(s, d2_64f(A[i].x, A[i].y, B[i].x, B[i].y));
        v = s;
      }
    } else if (n > 0 && m > 0) {
      const double h1 = warp_directed64(A, n, B, m), h2 = warp_directed64(B, m, A, n);
      v = h1 > h2 ? h1 : h2;
    }
    if (lane == 0) a.out64[w] = v;
  }
}

int launch_pw(tsim_ctx* ctx, void (*kern)(PwArgs), const PwArgs& a) {
  if (a.npairs <= 0) return TSIM_OK;
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPwThreads, 0));
  const long long warps = kPwThreads / 32;
  long long blocks = std::min<long long>((a.npairs + warps - 1) / warps,
                                         (long long)std::max(per_sm, 1) * ctx->num_sms);
  kern<<<(unsigned)std::max(blocks, 1ll), kPwThreads, 0, ctx->stream>>>(a);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

}  // namespace

int launch_pairwise(tsim_ctx* ctx, int measure, const PwArgs& a) {
  return launch_pw(ctx, measure == TSIM_HAUSDORFF ? hausdorff_refine_kernel : euclid_refine_kernel,
                   a);
}

int launch_pairwise64(tsim_ctx* ctx, int measure, const PwArgs& a) {
  if (a.npairs <= 0) return TSIM_OK;
  int per_sm = 0;
  TSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pairwise64_kernel, kPwThreads, 0));
  const long long warps = kPwThreads / 32;
  long long blocks = std::min<long long>((a.npairs + warps - 1) / warps,
                                         (long long)std::max(per_sm, 1) * ctx->num_sms);
  pairwise64_kernel<<<(unsigned)std::max(blocks, 1ll), kPwThreads, 0, ctx->stream>>>(
      a, measure == TSIM_EUCLIDEAN ? 1 : 0);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  return TSIM_OK;
}

}  // namespace tsim
