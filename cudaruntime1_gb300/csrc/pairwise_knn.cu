// pairwise_knn.cu -- exact kNN for symmetric Hausdorff and lock-step Euclidean.
#include "tsim_internal.cuh"

namespace tsim {

int knn_pairwise(tsim_ctx* ctx, const tsim_params* p, const float2* qpts, const int64_t* qoff,
                 int nq, int max_qlen, tsim_db* db, int* ids, float* dists, double* dists64,
                 tsim_stats* st) {
  (void)ctx; (void)p; (void)qpts; (void)qoff; (void)nq; (void)max_qlen; (void)db; (void)ids;
  (void)dists; (void)dists64; (void)st;
  return fail(TSIM_ERR_UNSUPPORTED, "Hausdorff/Euclidean kNN not built yet");
}

}  // namespace tsim
