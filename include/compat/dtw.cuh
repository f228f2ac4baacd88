// dtw.cuh -- drop-in for CudaRuntime1/dtw.cuh.
#ifndef DTW_CUH
#define DTW_CUH
#include "common.cuh"
// GPU path, implemented by libtsim.so (replaces CudaRuntime1/dtw.cu:99-234).
void launch_dtw_batch_gpu_knn(const Point* h_t1, const Point* h_t2, float* h_results, int num_t,
                              int n, int m, float& gpu_time);
// The reference's CPU baseline (CudaRuntime1/dtw.cpp:14); declared for source
// compatibility only, libtsim.so does not define it.
float launch_dtw_batch_cpu(const Point* h_t1, const Point* h_t2, float* h_results, int num_t,
                           int n, int m);
#endif
