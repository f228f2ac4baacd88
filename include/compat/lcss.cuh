// lcss.cuh -- drop-in for CudaRuntime1/lcss.cuh.
#ifndef LCSS_CUH
#define LCSS_CUH
#include "common.cuh"
// GPU path, implemented by libtsim.so (replaces CudaRuntime1/lcss.cu:114-250).
void launch_lcss_batch_gpu_wavefront_knn(const Point* h_t1, const Point* h_t2, float* h_results,
                                         int num_t, int n, int m, float epsilon, float& gpu_time);
// The reference's CPU baseline (CudaRuntime1/lcss.cpp:13); declared only.
float launch_lcss_batch_cpu(const Point* h_t1, const Point* h_t2, float* h_results, int num_t,
                            int n, int m, float epsilon);
#endif
