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

// Extract the K smallest packed keys of keys[0..N) in ascending order into
// out[0..K) (~0 when fewer than K remain).  Keys must be unique; each
// extracted key is overwritten with ~0 by the thread that owns its slot.
__device__ inline void block_select_k(unsigned long long* keys, int N, int K,
                                      unsigned long long* out, unsigned long long* red) {
  for (int k = 0; k < K; ++k) {
    unsigned long long best = ~0ull;
    int bpos = -1;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      unsigned long long x = keys[i];
      if (x < best) {
        best = x;
        bpos = i;
      }
    }
    const unsigned long long g = block_min_u64(best, red);
    if (g != ~0ull && best == g) keys[bpos] = ~0ull;
    if (threadIdx.x == 0) out[k] = g;
    __syncthreads();
  }
}

__device__ __forceinline__ int key_index(unsigned long long key) {
  return key == ~0ull ? -1 : (int)(key & 0xffffffffu);
}

}  // namespace tsim
