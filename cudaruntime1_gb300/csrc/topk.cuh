// topk.cuh -- block-level k-smallest selection over (key, index) pairs.
//
// Keys are packed as (order-preserving float bits << 32 | index), so the
// unsigned 64-bit minimum is the smallest key with ties broken by the
// smallest index: the order std::partial_sort gives the reference's
// std::vector<std::pair<float,int>> (CudaRuntime1/dtw.cpp:62) and the order a
// descending std::stable_sort gives after negating the key (lcss.cpp:67-70).
#pragma once
#include "tsim_internal.cuh"

namespace tsim {

__device__ __forceinline__ unsigned long long pack_key(float key, int idx) {
  return ((unsigned long long)f2ord(key) << 32) | (unsigned)idx;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
  for (int o = 16; o; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Block-wide minimum; `red` is shared scratch of >= 33 entries.  All threads
// of the block must call it; everyone gets the result.
__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long v,
                                                            unsigned long long* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  v = warp_min_u64(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    unsigned long long x = lane < nwarps ? red[lane] : ~0ull;
    x = warp_min_u64(x);
    if (lane == 0) red[32] = x;
  }
  __syncthreads();
  unsigned long long r = red[32];
  __syncthreads();
  return r;
}

// Shared scratch of block_select_k.
struct SelScratch {
  int hist[256];
  unsigned long long cand[64];
  unsigned long long pfx;  // digits of the K-th smallest key fixed so far
  int need;                // keys still to take at and above the current digit
  int shift;               // bit position of the last digit fixed
  int cnt;
  int stop;                // 1: the keys up to pfx at `shift` are the K; 2: all keys
};

// The K (<= 64) smallest packed keys of keys[0..N) (unique; ~0 = absent) in
// ascending order into out[0..K) (~0 when fewer than K are present).  All
// threads of the block must call it; out is visible to all on return.
// Radix selection from the top 8-bit digit down: a histogram of the keys
// that share the digits fixed so far locates the digit of the K-th smallest
// key; it stops when that digit's bin holds exactly the keys still needed
// (unique keys: at the last digit at the latest), then the at most K keys
// at or below that prefix are collected and ranked.
__device__ inline void block_select_k(const unsigned long long* keys, int N, int K,
                                      unsigned long long* out, SelScratch& S) {
  if (K <= 0) return;
  if (K <= 4) {  // a few block minima cost less than the digit passes
    unsigned long long prev = 0ull;
    for (int k = 0; k < K; ++k) {
      unsigned long long best = ~0ull;
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const unsigned long long x = keys[i];
        if ((k == 0 || x > prev) && x < best) best = x;
      }
      prev = block_min_u64(best, S.cand);
      if (threadIdx.x == 0) out[k] = prev;
    }
    __syncthreads();
    return;
  }
  if (threadIdx.x == 0) {
    S.pfx = 0;
    S.need = K;
    S.stop = 0;
    S.shift = 64;
  }
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) S.hist[i] = 0;
    __syncthreads();  // also publishes the previous pass's prefix
    const unsigned long long pfx = S.pfx;
    const int hs = shift + 8;
    // warp-aggregated counts: most keys share a few bins of the top digits
    for (int b = 0; b < N; b += blockDim.x) {
      const int i = b + threadIdx.x;
      const unsigned long long x = i < N ? keys[i] : ~0ull;
      const bool in = x != ~0ull && (hs >= 64 || (x >> hs) == (pfx >> hs));
      const unsigned bin = in ? (unsigned)(x >> shift) & 255u : 256u;
      const unsigned same = __match_any_sync(0xffffffffu, bin);
      if (in && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&S.hist[bin], __popc(same));
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      int c[8], sum = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        c[j] = S.hist[lane * 8 + j];
        sum += c[j];
      }
      int inc = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      const int total = __shfl_sync(0xffffffffu, inc, 31);
      const int need = S.need;
      if (total < need) {  // fewer keys than K at all (first pass only)
        if (lane == 0) S.stop = 2;
      } else if (inc - sum < need && need <= inc) {  // the lane holding the need-th key
        int run = inc - sum, d = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (run + c[j] >= need) {
            d = j;
            break;
          }
          run += c[j];
        }
        const int bin = c[d];
        S.pfx = pfx | ((unsigned long long)(lane * 8 + d) << shift);
        S.need = need - run;
        S.shift = shift;
        if (bin == need - run) S.stop = 1;
      }
    }
    __syncthreads();
    if (S.stop) break;
  }
  const int stop = S.stop, sh = S.shift;
  const unsigned long long lim = sh < 64 ? S.pfx >> sh : 0ull;
  if (threadIdx.x == 0) S.cnt = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const unsigned long long x = keys[i];
    if (x == ~0ull || (stop != 2 && (x >> sh) > lim)) continue;
    const int p = atomicAdd(&S.cnt, 1);
    if (p < 64) S.cand[p] = x;
  }
  __syncthreads();
  const int cnt = min(min(S.cnt, K), 64);
  for (int t = threadIdx.x; t < K; t += blockDim.x) {
    if (t < cnt) {
      const unsigned long long x = S.cand[t];
      int r = 0;
      for (int j = 0; j < cnt; ++j) r += S.cand[j] < x ? 1 : 0;
      out[r] = x;
    } else {
      out[t] = ~0ull;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int key_index(unsigned long long key) {
  return key == ~0ull ? -1 : (int)(key & 0xffffffffu);
}

}  // namespace tsim
