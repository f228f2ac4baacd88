// euclidean.cuh -- drop-in for CudaRuntime1/euclidean.cuh.
#ifndef EUCLIDEAN_CUH
#define EUCLIDEAN_CUH
#include "common.cuh"
// The reference's CPU baseline (CudaRuntime1/euclidean.cpp:43, needs Boost);
// declared only.
float launch_euclidean_batch_cpu_rtree(const Point* h_t1, const Point* h_t2, float* h_results,
                                       int num_t, int n);
// GPU pipeline, implemented by libtsim.so (replaces
// CudaRuntime1/euclidean_rtree.cpp:19-93): the 50 nearest bounding boxes
// per query on the GPU, then the exact lock-step distance; gpu_time = total ms.
void launch_euclidean_batch_gpu_rtree_exact(const Point* h_t1, const Point* h_t2,
                                            float* h_results, int num_t, int n, float& gpu_time);
// GPU kernel over caller-given CSR candidates (replaces
// CudaRuntime1/euclidean.cu:75-117); gpu_time = kernel time in ms.
void execute_rtree_csr_kernel_on_gpu(const Point* h_t1, const Point* h_t2, const int* h_candidates,
                                     const int* h_offsets, float* h_results, int num_t, int n,
                                     int total_candidates, float& gpu_time);
#endif
