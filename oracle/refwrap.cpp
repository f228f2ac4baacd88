// refwrap.cpp -- C entry points onto the reference's own CPU functions.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with the
// reference's CudaRuntime1/dtw.cpp, lcss.cpp and frechet.cpp, read in place
// from the reference checkout, into oracle/_ref/libref.so.  Used to pin the
// oracle's restatements (oracle.c) and to generate tests/golden fixtures.
// hausdorff.cpp, hausdorff_rtree.cpp, euclidean.cpp and euclidean_rtree.cpp
// need Boost.Geometry, which is not installed, so they are not built.
#include "dtw.cuh"      // CudaRuntime1/dtw.cuh:7
#include "lcss.cuh"     // CudaRuntime1/lcss.cuh:8
#include "frechet.cuh"  // CudaRuntime1/frechet.cuh:8

extern "C" {
float ref_dtw_cpu(const float* t1, const float* t2, float* out, int num_t, int n, int m) {
  return launch_dtw_batch_cpu(reinterpret_cast<const Point*>(t1),
                              reinterpret_cast<const Point*>(t2), out, num_t, n, m);
}
float ref_lcss_cpu(const float* t1, const float* t2, float* out, int num_t, int n, int m,
                   float eps) {
  return launch_lcss_batch_cpu(reinterpret_cast<const Point*>(t1),
                               reinterpret_cast<const Point*>(t2), out, num_t, n, m, eps);
}
float ref_frechet_cpu(const float* t1, const float* t2, float* out, int num_t, int n, int m) {
  return launch_frechet_batch_cpu(reinterpret_cast<const Point*>(t1),
                                  reinterpret_cast<const Point*>(t2), out, num_t, n, m);
}
}
