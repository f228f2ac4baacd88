// debug_bounds.cuh -- index checks for shared-memory accesses in the
// TSIM_DEBUG_BOUNDS build (libtsim_debug.so), the stand-in for a memory
// checker that cannot run here.
//
// TSIM_SIDX(i, cap) is the index i of a shared-memory array of cap elements.
// In the debug build an index outside [0, cap) is counted in this
// translation unit's device counter, its first value and capacity recorded,
// and 0 is used instead, so the kernel carries on without touching memory
// outside the array (no trap, no fault).  In the product build it is i.
// tsim_debug_bounds_violations (capi.cu) sums the counters of every
// translation unit that registers its reader with TSIM_BOUNDS_READER.
#pragma once
#include "tsim_internal.cuh"

namespace tsim {
// one reader per translation unit: adds the unit's count to *n, returns a CUDA error
using BoundsReader = cudaError_t (*)(unsigned long long* n, long long* first_bad);
int register_bounds_reader(BoundsReader r);
}  // namespace tsim

#ifdef TSIM_DEBUG_BOUNDS
namespace {
__device__ unsigned long long g_bounds_count;
__device__ long long g_bounds_first;  // (index << 32) | capacity of the first violation

__device__ __forceinline__ int tsim_checked_index(long long i, long long cap) {
  if (i >= 0 && i < cap) return (int)i;
  if (atomicAdd(&g_bounds_count, 1ull) == 0ull)
    g_bounds_first = (long long)((unsigned long long)(i & 0xffffffffll) << 32 | (unsigned)cap);
  return 0;
}

cudaError_t read_bounds(unsigned long long* n, long long* first_bad) {
  unsigned long long c = 0;
  long long f = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&c, g_bounds_count, sizeof(c));
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&f, g_bounds_first, sizeof(f));
  if (e == cudaSuccess && c) {
    if (*n == 0) *first_bad = f;
    *n += c;
  }
  return e;
}
const int g_bounds_registered = tsim::register_bounds_reader(read_bounds);
}  // namespace
#define TSIM_SIDX(i, cap) tsim_checked_index((long long)(i), (long long)(cap))
#else
#define TSIM_SIDX(i, cap) (i)
#endif
