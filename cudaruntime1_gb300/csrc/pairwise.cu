// pairwise.cu -- tiled pairwise-distance reductions: symmetric Hausdorff
// (max-min), lock-step Euclidean (sum), and the bounding-box candidate
// generator that stands in for the reference's Boost R-tree.
#include "debug_bounds.cuh"
#include "topk.cuh"
#include "tsim_internal.cuh"

namespace tsim {

// squared point distance without FMA: the reference CPU arithmetic
// (hausdorff.cpp:77-79), so values match it bit for bit
__device__ __forceinline__ float d2_exact(float ax, float ay, float bx, float by) {
  float dx = ax - bx, dy = ay - by;
  return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

namespace {

constexpr int kHdThreads = 256;

// max over a in S of min over b in T of |a-b|^2, S and T in shared memory,
// every thread of the CTA busy: with ns < kHdThreads sources, P threads
// (P = ns rounded up to a power of two, at least a warp) take the sources
// and the kHdThreads / P groups split the targets, their minima meeting in
// shared memory (red: kHdThreads floats).  Minimum and maximum are exact in
// any order, so the value is the sequential loop's.
__device__ float directed_max_min(const float2* S, int ns, const float2* T, int nt, float* red) {
  int P = 32;
  while (P < ns && P < kHdThreads) P <<= 1;
  const int G = kHdThreads / P;  // target groups
  const int g = threadIdx.x / P, il = threadIdx.x % P;
  float run = 0.0f;
  for (int base = 0; base < ns; base += P) {
    const int i = base + il;
    const float2 a = S[TSIM_SIDX(i < ns ? i : 0, ns)];
    float mn = TSIM_INF;
    int j = g;
    for (; j + 3 * G < nt; j += 4 * G) {  // four independent targets per iteration
      const float2 b0 = T[TSIM_SIDX(j, nt)], b1 = T[TSIM_SIDX(j + G, nt)],
                   b2 = T[TSIM_SIDX(j + 2 * G, nt)], b3 = T[TSIM_SIDX(j + 3 * G, nt)];
      mn = fminf(mn, fminf(fminf(d2_exact(a.x, a.y, b0.x, b0.y), d2_exact(a.x, a.y, b1.x, b1.y)),
                           fminf(d2_exact(a.x, a.y, b2.x, b2.y), d2_exact(a.x, a.y, b3.x, b3.y))));
    }
    for (; j < nt; j += G) {
      const float2 b = T[TSIM_SIDX(j, nt)];
      mn = fminf(mn, d2_exact(a.x, a.y, b.x, b.y));
    }
    red[threadIdx.x] = mn;
    __syncthreads();
    float loc = 0.0f;
    if (threadIdx.x < P && base + (int)threadIdx.x < ns) {
      float m2 = red[threadIdx.x];
      for (int h = 1; h < G; ++h) m2 = fminf(m2, red[TSIM_SIDX(h * P + threadIdx.x, kHdThreads)]);
      loc = m2;
    }
    for (int o = 16; o; o >>= 1) loc = fmaxf(loc, __shfl_xor_sync(0xffffffffu, loc, o));
    __syncthreads();  // red is reused below
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loc;
    __syncthreads();
    for (int w = 0; w < kHdThreads / 32; ++w) run = fmaxf(run, red[w]);
    __syncthreads();
  }
  return run;
}

// One CTA per query: the query in shared memory once, its top_k candidates
// in turn (the reference's hausdorff_tiled_rtree_kernel order,
// CudaRuntime1/hausdorff.cu:84-122); symmetric Hausdorff^2 =
// max(h(A,B), h(B,A)), the second direction skipped once the first already
// exceeds the query's best.
__global__ void __launch_bounds__(kHdThreads)
    hausdorff_cands_kernel(const float2* __restrict__ t1, int n, const float2* __restrict__ t2,
                           int num_t2, int m, const int* __restrict__ cand, int top_k,
                           unsigned* __restrict__ best_bits) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float red[kHdThreads];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  float2* B = A + n;
  const int q = blockIdx.x;
  const float2* ga = t1 + (size_t)q * n;
  for (int i = threadIdx.x; i < n; i += kHdThreads) A[TSIM_SIDX(i, n)] = ga[i];
  float best = TSIM_INF;
  for (int k = 0; k < top_k; ++k) {
    const int c = cand[(size_t)q * top_k + k];
    if (c < 0 || c >= num_t2) continue;  // out-of-range candidate slots are ignored
    const float2* gb = t2 + (size_t)c * m;
    __syncthreads();  // the previous candidate is done with B
    for (int i = threadIdx.x; i < m; i += kHdThreads) B[TSIM_SIDX(i, m)] = gb[i];
    __syncthreads();
    const float h1 = directed_max_min(A, n, B, m, red);
    if (!(h1 < best)) continue;  // uniform: every thread holds the same h1
    const float h = fmaxf(h1, directed_max_min(B, m, A, n, red));
    best = fminf(best, h);
  }
  if (threadIdx.x == 0) best_bits[q] = __float_as_uint(best);
}

__global__ void sqrt_bits_kernel(const unsigned* bits, float* out, int count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = __fsqrt_rn(__uint_as_float(bits[i]));
}

// ---- lock-step Euclidean -----------------------------------------------------
constexpr int kEuThreads = 128;

// TwoSum: s + e == a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Warp per query (the reference's block per query, CudaRuntime1/euclidean.cu:
// 17-73).  First its CSR entries four at a time, 8 lanes each: compensated
// FP32 sums of squared point differences (TwoSum per lane, a compensated
// butterfly over the 8); their order does not matter, since they only pick
// the candidates whose sum lies within its rigorous error margin of the
// smallest.  Those are re-scored in FP64 left to right exactly like
// calc_exact_dist_sq (euclidean.cpp:27-40): the lanes compute 32 terms
// dx^2 + dy^2 at a time, and every lane adds them to the running sum in
// point order; out = (float)sqrt of the best.
__global__ void __launch_bounds__(kEuThreads)
    euclid_cands_kernel(const float2* __restrict__ t1, const float2* __restrict__ t2,
                        const int* __restrict__ cand, const int* __restrict__ off, int num_t, int n,
                        int total, float* __restrict__ s32, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= num_t) return;
  // clamp caller offsets into [0, total] so a malformed CSR cannot read out of bounds
  const int b = min(max(off[q], 0), total), e = max(min(off[q + 1], total), b);
  const float2* A = t1 + (size_t)q * n;
  const int grp = lane >> 3, gl = lane & 7;
  float mn = TSIM_INF;
  for (int base = b; base < e; base += 4) {
    const int idx = base + grp;
    const int ce = idx < e ? cand[idx] : -1;
    const bool ok = ce >= 0 && ce < num_t;  // out-of-range candidates never win
    const float2* B = t2 + (size_t)(ok ? ce : 0) * n;
    float sum = 0.0f, c = 0.0f;
    for (int i = gl; i < n; i += 8) {
      const float2 p = A[i], r = B[i];
      const float dx = p.x - r.x, dy = p.y - r.y;
      float ns, err;
      two_sum(sum, fmaf(dy, dy, dx * dx), ns, err);
      sum = ns;
      c += err;
    }
    for (int o = 4; o; o >>= 1) {
      const float s2 = __shfl_xor_sync(0xffffffffu, sum, o);
      const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
      float ns, err;
      two_sum(sum, s2, ns, err);
      sum = ns;
      c = c + c2 + err;
    }
    const float tot = ok ? sum + c : TSIM_INF;
    if (gl == 0 && idx < e) s32[idx] = tot;
    mn = fminf(mn, tot);
  }
  for (int o = 16; o >= 8; o >>= 1) mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  __syncwarp();
  // |s32 - exact| <= g * exact with g = 2^-20 (terms 2u, TwoSum chain ~2u,
  // final fold ~2u, n*u^2 negligible for n < 2^20)
  const double g = 1.0 / (1 << 20);
  const double thr = (double)mn * (1.0 + g) / (1.0 - g);
  double best = 1.7976931348623157e308;
  for (int base = b; base < e; base += 32) {
    const int idx = base + lane;
    bool need = false;
    if (idx < e) need = (double)s32[idx] <= thr && cand[idx] >= 0 && cand[idx] < num_t;
    unsigned todo = __ballot_sync(0xffffffffu, need);
    while (todo) {
      const int l = __ffs(todo) - 1;
      todo &= todo - 1;
      const float2* B = t2 + (size_t)cand[base + l] * n;
      double s = 0.0;
      for (int k0 = 0; k0 < n; k0 += 32) {
        double t = 0.0;
        if (k0 + lane < n) {
          const double dx = (double)A[k0 + lane].x - (double)B[k0 + lane].x;
          const double dy = (double)A[k0 + lane].y - (double)B[k0 + lane].y;
          t = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        }
        const int cnt = min(32, n - k0);
        for (int u = 0; u < cnt; ++u) s = __dadd_rn(s, __shfl_sync(0xffffffffu, t, u));
      }
      best = s < best ? s : best;
    }
  }
  if (lane == 0) out[q] = __double2float_rn(__dsqrt_rn(best));
}

// ---- bounding boxes and box nearest neighbours --------------------------------
__global__ void boxes_kernel(const float2* __restrict__ t, int count, int len,
                             float4* __restrict__ box) {
  const int lane = threadIdx.x & 31;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= count) return;
  const float2* p = t + (size_t)w * len;
  // sequential min/max semantics do not matter for the value of a min/max
  float x0 = TSIM_INF, y0 = TSIM_INF, x1 = -TSIM_INF, y1 = -TSIM_INF;
  for (int i = lane; i < len; i += 32) {
    float2 v = p[i];
    x0 = fminf(x0, v.x);
    x1 = fmaxf(x1, v.x);
    y0 = fminf(y0, v.y);
    y1 = fmaxf(y1, v.y);
  }
  for (int o = 16; o; o >>= 1) {
    x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
  }
  if (lane == 0) box[w] = make_float4(x0, y0, x1, y1);
}

__device__ __forceinline__ float smaxf(float a, float b) { return (a < b) ? b : a; }

__device__ __forceinline__ float box_box_d2(float4 a, float4 b) {
  float dx = smaxf(0.0f, smaxf(__fsub_rn(a.x, b.z), __fsub_rn(b.x, a.z)));
  float dy = smaxf(0.0f, smaxf(__fsub_rn(a.y, b.w), __fsub_rn(b.y, a.w)));
  return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

constexpr int kSelThreads = 256;

__global__ void __launch_bounds__(kSelThreads)
    mbr_knn_kernel(const float4* __restrict__ qbox, const float4* __restrict__ cbox, int num_t2,
                   int k, unsigned long long* __restrict__ gkeys, int* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SelScratch red;
  const int q = blockIdx.x;
  unsigned long long* keys =
      gkeys ? gkeys + (size_t)q * num_t2 : reinterpret_cast<unsigned long long*>(smem_raw);
  unsigned long long* sel =
      reinterpret_cast<unsigned long long*>(smem_raw + (gkeys ? 0 : (size_t)num_t2 * 8));
  const float4 a = qbox[q];
  for (int j = threadIdx.x; j < num_t2; j += kSelThreads) keys[j] = pack_key(box_box_d2(a, cbox[j]), j);
  __syncthreads();
  block_select_k(keys, num_t2, min(k, num_t2), sel, red);
  const int got = min(k, num_t2);
  for (int e = threadIdx.x; e < k; e += kSelThreads)
    out[(size_t)q * k + e] = e < got ? key_index(sel[e]) : (got > 0 ? key_index(sel[got - 1]) : 0);
}

}  // namespace

int hausdorff_cands(tsim_ctx* ctx, const float2* t1, int num_t1, int n, const float2* t2, int num_t2,
                    int m, const int* cand, int top_k, float* out) {
  TSIM_TRY(arena_reserve(ctx, align256(sizeof(unsigned) * num_t1)));
  unsigned* best = arena_take<unsigned>(ctx, num_t1);
  size_t smem = sizeof(float2) * ((size_t)n + m);
  TSIM_CHECK_ARG(smem <= 200 * 1024, "trajectories too long for the shared-memory Hausdorff kernel");
  if (smem > 48 * 1024)
    TSIM_CUDA(cudaFuncSetAttribute(hausdorff_cands_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  hausdorff_cands_kernel<<<num_t1, kHdThreads, smem, ctx->stream>>>(t1, n, t2, num_t2, m, cand,
                                                                     top_k, best);
  sqrt_bits_kernel<<<(num_t1 + 255) / 256, 256, 0, ctx->stream>>>(best, out, num_t1);
  TSIM_CUDA(cudaGetLastError());
  return TSIM_OK;
}

int euclid_cands(tsim_ctx* ctx, const float2* t1, const float2* t2, const int* cand, const int* off,
                 int num_t, int n, int total, float* out) {
  TSIM_TRY(arena_reserve(ctx, align256(sizeof(float) * std::max(total, 1))));
  float* s32 = arena_take<float>(ctx, std::max(total, 1));
  const int warps = kEuThreads / 32;
  euclid_cands_kernel<<<(num_t + warps - 1) / warps, kEuThreads, 0, ctx->stream>>>(
      t1, t2, cand, off, num_t, n, total, s32, out);
  TSIM_CUDA(cudaGetLastError());
  return TSIM_OK;
}

int mbr_knn(tsim_ctx* ctx, const float2* t1, int num_t1, int n, const float2* t2, int num_t2, int m,
            int k, int* out) {
  size_t key_bytes = sizeof(unsigned long long) * (size_t)num_t2;
  bool in_smem = key_bytes + 64 * sizeof(unsigned long long) <= 200 * 1024;
  size_t need = align256(sizeof(float4) * num_t1) + align256(sizeof(float4) * num_t2) +
                (in_smem ? 0 : align256(key_bytes * num_t1) + align256((size_t)k * 4 * num_t1));
  TSIM_TRY(arena_reserve(ctx, need));
  float4* qb = arena_take<float4>(ctx, num_t1);
  float4* cb = arena_take<float4>(ctx, num_t2);
  unsigned long long* gkeys = in_smem ? nullptr : arena_take<unsigned long long>(ctx, (size_t)num_t2 * num_t1);
  boxes_kernel<<<(num_t1 + 3) / 4, 128, 0, ctx->stream>>>(t1, num_t1, n, qb);
  boxes_kernel<<<(num_t2 + 3) / 4, 128, 0, ctx->stream>>>(t2, num_t2, m, cb);
  size_t smem = (in_smem ? key_bytes : 0) + 64 * sizeof(unsigned long long);
  TSIM_CUDA(cudaFuncSetAttribute(mbr_knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  mbr_knn_kernel<<<num_t1, kSelThreads, smem, ctx->stream>>>(qb, cb, num_t2, k, gkeys, out);
  TSIM_CUDA(cudaGetLastError());
  return TSIM_OK;
}

}  // namespace tsim

extern "C" {

int tsim_hausdorff_cands(tsim_ctx* ctx, const tsim_point* d_t1, int num_t1, int n,
                         const tsim_point* d_t2, int num_t2, int m, const int* d_cand, int top_k,
                         float* d_out) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  TSIM_CHECK_ARG(num_t1 >= 1 && num_t2 >= 1 && n >= 1 && m >= 1 && top_k >= 1, "sizes must be >= 1");
  TSIM_CHECK_ARG(d_t1 && d_t2 && d_cand && d_out, "NULL device pointer");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  return tsim::hausdorff_cands(ctx, (const float2*)d_t1, num_t1, n, (const float2*)d_t2, num_t2, m,
                               d_cand, top_k, d_out);
}

int tsim_euclid_cands(tsim_ctx* ctx, const tsim_point* d_t1, const tsim_point* d_t2,
                      const int* d_cand, const int* d_off, int num_t, int n, int total,
                      float* d_out) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  TSIM_CHECK_ARG(num_t >= 1 && n >= 1 && total >= 0, "bad sizes");
  TSIM_CHECK_ARG(d_t1 && d_t2 && d_off && d_out && (total == 0 || d_cand), "NULL device pointer");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  return tsim::euclid_cands(ctx, (const float2*)d_t1, (const float2*)d_t2, d_cand, d_off, num_t, n,
                            total, d_out);
}

int tsim_mbr_knn(tsim_ctx* ctx, const tsim_point* d_t1, int num_t1, int n, const tsim_point* d_t2,
                 int num_t2, int m, int k, int* d_out) {
  TSIM_CHECK_ARG(ctx != nullptr, "ctx is NULL");
  TSIM_CHECK_ARG(num_t1 >= 1 && num_t2 >= 1 && n >= 1 && m >= 1 && k >= 1 && k <= 64,
                 "sizes must be >= 1 and k <= 64");
  TSIM_CHECK_ARG(d_t1 && d_t2 && d_out, "NULL device pointer");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  return tsim::mbr_knn(ctx, (const float2*)d_t1, num_t1, n, (const float2*)d_t2, num_t2, m, k, d_out);
}

}  // extern "C"
