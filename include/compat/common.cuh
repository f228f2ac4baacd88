// common.cuh -- drop-in for CudaRuntime1/common.cuh (lines 1-23): the Point
// type and the CHECK macro that the reference's callers use.  Point has the
// same 8-byte layout as tsim_point in include/tsim.h.
#ifndef COMMON_CUH
#define COMMON_CUH

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

struct Point {
  float x, y;
};

// Caller-side convenience kept for source compatibility: prints the CUDA
// error and exits, as the reference's macro does (common.cuh:14-22).  The
// library itself never uses it.
#define CHECK(call)                                                           \
  do {                                                                        \
    const cudaError_t error = call;                                           \
    if (error != cudaSuccess) {                                               \
      printf("Error: %s:%d, ", __FILE__, __LINE__);                           \
      printf("code: %d, reason: %s\n", error, cudaGetErrorString(error));     \
      exit(1);                                                                \
    }                                                                         \
  } while (0)

#endif
