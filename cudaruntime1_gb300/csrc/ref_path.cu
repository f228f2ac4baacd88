// ref_path.cu -- reference-semantics batch path for DTW, LCSS and Frechet.
//
// The reference (CudaRuntime1/dtw.cu:99-234, lcss.cu:114-250,
// frechet.cu:120-253) builds the r=5 query envelopes on the host, computes a
// full num_t x num_t bound matrix on the GPU, copies it back, selects the
// K=10 best candidates per query with partial_sort on the host, copies the
// pair list in again, refines on the GPU and reduces on the host.
//
// Here everything after the H2D copy of the trajectories stays on the device:
//   1. ref_filter_kernel: one CTA per query builds the envelope in shared
//      memory, evaluates the bound of every candidate (summed in the same
//      order as the reference CPU code, so values are bit-identical), and
//      selects the K best by (bound, index) without materialising the matrix;
//   2. the wavefront DP kernel (dp_kernels.cu) refines the num_t*K pairs;
//   3. ref_reduce_kernel keeps the best refined value per query.
// Outputs equal the reference's CPU functions (dtw.cpp:14-113,
// lcss.cpp:13-115, frechet.cpp:13-124) bit for bit.
#include "topk.cuh"
#include "tsim_internal.cuh"

namespace tsim {
namespace {

constexpr int kFilterThreads = 256;
constexpr float kRefBig = 1e20f;  // the reference's infinity (dtw.cpp:23)
constexpr size_t kRefSmemCap = 200 * 1024;

__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

// kind: 0 = DTW (sum of envelope distances), 1 = LCSS (eps-box count,
// descending), 2 = Frechet (max of envelope distances).
template <int KIND>
__global__ void __launch_bounds__(kFilterThreads)
    ref_filter_kernel(const float2* __restrict__ t1, const float2* __restrict__ t2, int num_t,
                      int n, int m, float eps, int K, unsigned long long* __restrict__ gkeys,
                      int2* __restrict__ pairs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SelScratch red;
  const int q = blockIdx.x;
  // envelope of query point v*n/m for each candidate position v, m entries
  float4* envv = reinterpret_cast<float4*>(smem_raw);
  unsigned long long* keys =
      gkeys ? gkeys + (size_t)q * num_t : reinterpret_cast<unsigned long long*>(envv + m);
  const float2* A = t1 + (size_t)q * n;
  const int r = 5;
  for (int v = threadIdx.x; v < m; v += blockDim.x) {
    const int i = (int)(((long long)v * n) / m);
    float min_x = kRefBig, max_x = -kRefBig, min_y = kRefBig, max_y = -kRefBig;
    const int s = max(0, i - r), e = min(n - 1, i + r);
    for (int k = s; k <= e; ++k) {
      float2 p = A[k];
      min_x = smin(min_x, p.x);
      max_x = smax(max_x, p.x);
      min_y = smin(min_y, p.y);
      max_y = smax(max_y, p.y);
    }
    envv[v] = make_float4(min_x, max_x, min_y, max_y);
  }
  __syncthreads();
  const int min_len = min(n, m);
  for (int j = threadIdx.x; j < num_t; j += blockDim.x) {
    const float2* C = t2 + (size_t)j * m;
    float key;
    if (KIND == 1) {
      int cnt = 0;
      for (int v = 0; v < m; ++v) {
        const float4 e = envv[v];
        const float2 p = __ldg(C + v);
        if (p.x > __fsub_rn(e.x, eps) && p.x < __fadd_rn(e.y, eps) && p.y > __fsub_rn(e.z, eps) &&
            p.y < __fadd_rn(e.w, eps))
          cnt++;
      }
      key = -__fdiv_rn((float)cnt, (float)min_len);  // descending ub -> ascending key
    } else {
      float acc = 0.0f;
      for (int v = 0; v < m; ++v) {
        const float4 e = envv[v];
        const float2 p = __ldg(C + v);
        float dx = smax(0.0f, smax(__fsub_rn(e.x, p.x), __fsub_rn(p.x, e.y)));
        float dy = smax(0.0f, smax(__fsub_rn(e.z, p.y), __fsub_rn(p.y, e.w)));
        float d = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
        acc = (KIND == 0) ? __fadd_rn(acc, d) : smax(acc, d);
      }
      key = acc;
    }
    keys[j] = pack_key(key, j);
  }
  __syncthreads();
  __shared__ unsigned long long sel[64];
  block_select_k(keys, num_t, K, sel, red);
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    pairs[(size_t)q * K + k] = make_int2(q, key_index(sel[k]));
}

// kind 0/2: min of refined distances; 1: max of count / min(n, m).
template <int KIND>
__global__ void ref_reduce_kernel(const float* __restrict__ vals, int num_t, int K, int n, int m,
                                  float* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= num_t) return;
  if (KIND == 1) {
    float best = -1.0f;
    const int min_len = min(n, m);
    for (int k = 0; k < K; ++k) {
      float sim = __fdiv_rn(vals[(size_t)q * K + k], (float)min_len);
      if (sim > best) best = sim;
    }
    out[q] = best;
  } else {
    float best = kRefBig;
    for (int k = 0; k < K; ++k) {
      float v = vals[(size_t)q * K + k];
      if (v < best) best = v;
    }
    out[q] = best;
  }
}

__global__ void fixed_offsets_kernel(int64_t* off, int count, int len) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= count) off[i] = (int64_t)i * len;
}

}  // namespace

// Scratch of one reference-semantics batch call, carved from one block.
size_t ref_scratch_bytes(int num_t, int m, bool* keys_in_smem) {
  const int K = std::min(10, num_t);
  const size_t env_bytes = (size_t)m * sizeof(float4);
  const size_t key_bytes = (size_t)num_t * sizeof(unsigned long long);
  const bool in_smem = env_bytes + key_bytes <= kRefSmemCap;
  if (keys_in_smem) *keys_in_smem = in_smem;
  return align256(sizeof(int2) * num_t * K) + align256(sizeof(float) * num_t * K) +
         2 * align256(sizeof(int64_t) * (num_t + 1)) + (in_smem ? 0 : align256(key_bytes * num_t));
}

int ref_batch_core(tsim_ctx* ctx, int measure, const float2* d_t1, const float2* d_t2, int num_t,
                   int n, int m, float eps, float* d_out, char* scratch) {
  const int K = std::min(10, num_t);
  // shared memory: m envelopes + keys when they fit, else keys in scratch
  const size_t env_bytes = (size_t)m * sizeof(float4);
  const size_t key_bytes = (size_t)num_t * sizeof(unsigned long long);
  TSIM_CHECK_ARG(env_bytes <= kRefSmemCap, "candidate length too large for the envelope filter");
  bool keys_in_smem = false;
  ref_scratch_bytes(num_t, m, &keys_in_smem);
  char* p = scratch;
  auto take = [&p](size_t bytes) {
    char* q = p;
    p += align256(bytes);
    return q;
  };
  int2* pairs = reinterpret_cast<int2*>(take(sizeof(int2) * num_t * K));
  float* vals = reinterpret_cast<float*>(take(sizeof(float) * num_t * K));
  int64_t* qoff = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (num_t + 1)));
  int64_t* coff = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (num_t + 1)));
  unsigned long long* gkeys =
      keys_in_smem ? nullptr : reinterpret_cast<unsigned long long*>(take(key_bytes * num_t));

  stage_begin(ctx, TSIM_STAGE_REF);
  const size_t smem = env_bytes + (keys_in_smem ? key_bytes : 0);
  auto launch_filter = [&](auto kern) -> int {
    if (smem > 48 * 1024)
      TSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<num_t, kFilterThreads, smem, ctx->stream>>>(d_t1, d_t2, num_t, n, m, eps, K, gkeys,
                                                        pairs);
    TSIM_CUDA(cudaGetLastError());
    launched(ctx);
    return TSIM_OK;
  };
  int kind;
  if (measure == TSIM_DTW) {
    TSIM_TRY(launch_filter(ref_filter_kernel<0>));
    kind = DP_DTW_REF;
  } else if (measure == TSIM_LCSS) {
    TSIM_TRY(launch_filter(ref_filter_kernel<1>));
    kind = DP_LCSS;
  } else {
    TSIM_TRY(launch_filter(ref_filter_kernel<2>));
    kind = DP_FRECHET_REF;
  }
  fixed_offsets_kernel<<<(num_t + 256) / 256, 256, 0, ctx->stream>>>(qoff, num_t, n);
  fixed_offsets_kernel<<<(num_t + 256) / 256, 256, 0, ctx->stream>>>(coff, num_t, m);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx, 2);

  DpArgs a{};
  a.qpts = d_t1;
  a.qoff = qoff;
  a.cpts = d_t2;
  a.coff = coff;
  a.pairs = pairs;
  a.npairs = num_t * K;
  a.out = vals;
  a.thr = nullptr;
  a.band_pct = -1;
  a.delta = -1;
  a.eps = eps;
  int G, R;
  dp_shape(kind, n, m, -1, G, R);
  TSIM_TRY(launch_dp(ctx, kind, G, R, a, m));

  const int tb = 128;
  if (measure == TSIM_LCSS)
    ref_reduce_kernel<1><<<(num_t + tb - 1) / tb, tb, 0, ctx->stream>>>(vals, num_t, K, n, m, d_out);
  else
    ref_reduce_kernel<0><<<(num_t + tb - 1) / tb, tb, 0, ctx->stream>>>(vals, num_t, K, n, m, d_out);
  TSIM_CUDA(cudaGetLastError());
  launched(ctx);
  stage_end(ctx);
  return TSIM_OK;
}

int ref_batch(tsim_ctx* ctx, int measure, const float2* d_t1, const float2* d_t2, int num_t, int n,
              int m, float eps, float* d_out) {
  TSIM_TRY(arena_reserve(ctx, ref_scratch_bytes(num_t, m, nullptr)));
  char* scratch = arena_take<char>(ctx, ref_scratch_bytes(num_t, m, nullptr));
  return ref_batch_core(ctx, measure, d_t1, d_t2, num_t, n, m, eps, d_out, scratch);
}

}  // namespace tsim

extern "C" int tsim_ref_batch(tsim_ctx* ctx, int measure, const tsim_point* d_t1,
                              const tsim_point* d_t2, int num_t, int n, int m, float epsilon,
                              float* d_out) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  TSIM_CHECK_ARG(measure == TSIM_DTW || measure == TSIM_LCSS || measure == TSIM_FRECHET,
                 "measure must be DTW, LCSS or Frechet");
  TSIM_CHECK_ARG(num_t >= 1 && n >= 1 && m >= 1, "num_t, n and m must be >= 1");
  TSIM_CHECK_ARG(d_t1 && d_t2 && d_out, "NULL device pointer");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  return tsim::ref_batch(ctx, measure, reinterpret_cast<const float2*>(d_t1),
                         reinterpret_cast<const float2*>(d_t2), num_t, n, m, epsilon, d_out);
}
