// hausdorff.cuh -- drop-in for CudaRuntime1/hausdorff.cuh.
#ifndef HAUSDORFF_CUH
#define HAUSDORFF_CUH
#include "common.cuh"
// The reference's CPU baseline (CudaRuntime1/hausdorff.cpp:137, needs Boost);
// declared only.
float launch_hausdorff_batch_cpu_rtree(const Point* h_t1, int num_t1, int n, const Point* h_t2,
                                       int num_t2, int m, float* h_results, int top_k = 10);
// GPU pipeline, implemented by libtsim.so (replaces
// CudaRuntime1/hausdorff_rtree.cpp:32-83): candidate generation by bounding-box
// nearest neighbours on the GPU instead of a host Boost R-tree.  Returns the
// total wall time in ms.
float run_hausdorff_rtree_gpu_pipeline(const Point* h_t1, int num_t1, int n, const Point* h_t2,
                                       int num_t2, int m, float* h_results, int top_k = 10);
// GPU kernel with caller-given candidates (replaces CudaRuntime1/hausdorff.cu:125-184);
// gpu_time = kernel time in ms.
void launch_hausdorff_rtree_gpu(const Point* h_t1, int num_t1, int n, const Point* h_t2,
                                int num_t2, int m, const int* h_candidate_indices, int top_k,
                                float* h_results, float& gpu_time);
#endif
