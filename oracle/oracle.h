/*
 * oracle.h -- CPU correctness oracle for the trajectory-similarity kNN path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by tests/, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py, always as the checker or the timed CPU
 * baseline, never as a fallback for the GPU path.
 *
 * Two families of functions:
 *
 *  1. orc_ref_*: restatements of the reference's own CPU functions
 *     (CudaRuntime1/dtw.cpp, lcss.cpp, frechet.cpp, hausdorff.cpp,
 *     euclidean.cpp), operation for operation in float so that results are
 *     bit-identical to the reference CPU code built without FP contraction.
 *     The DTW/LCSS/Frechet ones are pinned against the reference sources
 *     compiled into oracle/_ref (see oracle/Makefile) and against the golden
 *     fixtures in tests/golden.
 *
 *  2. orc_*64 / orc_knn: an FP64 brute-force exact kNN over all candidates,
 *     written from the definitions of the five measures, with ties broken by
 *     candidate index.  This is the reference for "bit-exact kNN ids" and
 *     "relative distance error" checks.
 *
 * Points are AoS float pairs (x, y), the layout of the reference's
 * `struct Point {float x, y;}` (CudaRuntime1/common.cuh:9-11).
 * Build with -ffp-contract=off: the reference was compiled for x86-64, where
 * `a*b + c` is never fused; on aarch64 GCC would fuse it by default.
 */
#ifndef TSIM_ORACLE_H
#define TSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_DTW = 0, ORC_LCSS = 1, ORC_FRECHET = 2, ORC_HAUSDORFF = 3, ORC_EUCLIDEAN = 4 };
enum { ORC_COST_SQEUCLID = 0, ORC_COST_EUCLID = 1 };

typedef struct {
  int measure;    /* ORC_* */
  int k;          /* neighbours per query */
  int cost;       /* DTW cell cost: ORC_COST_* */
  int band_pct;   /* DTW Sakoe-Chiba band, percent of max(n,m); <0 = no band */
  float epsilon;  /* LCSS per-coordinate match threshold (strict <) */
  int delta;      /* LCSS index window |i-j| <= delta; <0 = no window */
} orc_params;

/* ---- band geometry shared by oracle, filters and kernels ------------------ */
/* w = ceil(band_pct * max(n,m) / 100); -1 when band_pct < 0. */
int orc_band_w(int n, int m, int band_pct);
/* Columns j of row i inside |i*(m-1) - j*(n-1)| <= w*(min(n,m)-1).
 * Returns hi < lo for an empty row.  w < 0 means the whole row. */
void orc_band_row(int i, int n, int m, int w, int* lo, int* hi);

/* ---- 1. reference-semantics restatements (float) -------------------------- */
float orc_ref_dtw(const float* t1, const float* t2, float* out, int num_t, int n, int m);
float orc_ref_lcss(const float* t1, const float* t2, float* out, int num_t, int n, int m,
                   float epsilon);
float orc_ref_frechet(const float* t1, const float* t2, float* out, int num_t, int n, int m);
/* Grid-accelerated directed Hausdorff^2 with early break, seeded with a
 * running max (CudaRuntime1/hausdorff.cpp:11-109). */
float orc_ref_directed_hausdorff_grid(const float* src, int len_src, const float* tgt,
                                      int len_tgt, float seed_max_d2);
/* Min over the given candidates of the symmetric Hausdorff distance, as the
 * candidate loop of CudaRuntime1/hausdorff.cpp:164-182 computes it. */
void orc_ref_hausdorff_cands(const float* t1, int num_t1, int n, const float* t2, int num_t2,
                             int m, const int* cand, int top_k, float* out);
/* Min over CSR candidates of the FP64 lock-step distance with early abandon
 * (CudaRuntime1/euclidean.cpp:27-40, 86-113). */
void orc_ref_euclid_cands(const float* t1, const float* t2, const int* cand,
                          const int* offsets, float* out, int num_t, int n);
/* Replacement for the Boost R-tree `nearest(mbr, k)` candidate query: the k
 * trajectories whose bounding boxes are nearest (squared box-box distance in
 * float), ties by index, ascending.  Writes num_t1*k ints; pads like
 * CudaRuntime1/hausdorff_rtree.cpp:66-68 when num_t2 < k. */
void orc_mbr_knn(const float* t1, int num_t1, int n, const float* t2, int num_t2, int m, int k,
                 int* out);

/* ---- 2. FP64 exact measures and brute-force kNN --------------------------- */
double orc_dtw64(const float* a, int n, const float* b, int m, int band_pct, int cost);
int orc_lcss_count(const float* a, int n, const float* b, int m, float epsilon, int delta);
double orc_frechet64(const float* a, int n, const float* b, int m);
double orc_hausdorff64(const float* a, int n, const float* b, int m);
/* Lock-step Euclidean over the candidate's m points against the query's
 * first m points; +inf when the query is shorter than the candidate. */
double orc_euclid64(const float* q, int n, const float* c, int m);

/* Brute-force exact kNN.  ids[nq*k], dists[nq*k] (LCSS: the integer count
 * stored as a double).  Ranking: distance ascending (LCSS: count
 * descending), then candidate index ascending.  nthreads<=0: all cores. */
int orc_knn(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
            const float* dbpts, const int64_t* dboff, int ndb, int* ids, double* dists,
            int nthreads);

/* FP64 exact DTW kNN with lower-bound pruning (LB_Kim + banded LB_Keogh,
 * candidates in bound order, early abandon).  Same results as orc_knn for
 * measure DTW; used as the CPU baseline. */
int orc_dtw_knn_pruned(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
                       const float* dbpts, const int64_t* dboff, int ndb, int* ids,
                       double* dists, int nthreads, int64_t* cells_out);

/* Exact kNN with bound pruning for every measure: candidates visited in
 * order of an FP64 bound on their ranking key (DTW: banded LB_Keogh;
 * Frechet / Hausdorff: endpoints and point-to-box distances; LCSS: points
 * that could match the other's epsilon-inflated box; Euclidean: first and
 * last terms), in parallel chunks with early abandon against the k-th key.
 * Results equal orc_knn's, ties included; *evaluated (may be NULL) counts
 * the candidates whose exact value was computed. */
int orc_knn_pruned(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
                   const float* dbpts, const int64_t* dboff, int ndb, int* ids, double* dists,
                   int nthreads, int64_t* evaluated);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
