// frechet.cuh -- drop-in for CudaRuntime1/frechet.cuh.
#ifndef FRECHET_CUH
#define FRECHET_CUH
#include "common.cuh"
// GPU path, implemented by libtsim.so (replaces CudaRuntime1/frechet.cu:120-253).
void launch_frechet_batch_gpu_wavefront(const Point* h_t1, const Point* h_t2, float* h_results,
                                        int num_t, int n, int m, float& gpu_time);
// The reference's CPU baseline (CudaRuntime1/frechet.cpp:13); declared only.
float launch_frechet_batch_cpu(const Point* h_t1, const Point* h_t2, float* h_results, int num_t,
                               int n, int m);
#endif
