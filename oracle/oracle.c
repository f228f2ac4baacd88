/*
 * oracle.c -- CPU correctness oracle (TEST INFRASTRUCTURE ONLY; see oracle.h).
 *
 * Every reference-semantics function below restates one CPU function of
 * CudaRuntime1 operation for operation, in float, so its outputs equal the
 * reference's bit for bit when both are compiled without FP contraction.
 * The FP64 functions are written from the measures' definitions.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F_BIG 1e20f /* the reference's "infinity" (dtw.cpp:23, 65, 68) */

/* std::min / std::max exactly as libstdc++ defines them. */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* band geometry                                                              */
/* ------------------------------------------------------------------------- */

int orc_band_w(int n, int m, int band_pct) {
  if (band_pct < 0) return -1;
  int L = n > m ? n : m;
  return (int)(((long long)band_pct * L + 99) / 100);
}

static inline long long floordiv(long long a, long long b) {
  long long q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
  return q;
}
static inline long long ceildiv(long long a, long long b) { return -floordiv(-a, b); }

void orc_band_row(int i, int n, int m, int w, int* lo, int* hi) {
  if (w < 0 || n <= 1) {
    *lo = 0;
    *hi = m - 1;
    return;
  }
  long long mn = (n < m ? n : m) - 1;
  long long W = (long long)w * mn;
  long long c = (long long)i * (m - 1);
  long long l = ceildiv(c - W, n - 1), h = floordiv(c + W, n - 1);
  if (l < 0) l = 0;
  if (h > m - 1) h = m - 1;
  *lo = (int)l;
  *hi = (int)h;
}

/* ------------------------------------------------------------------------- */
/* 1. reference-semantics restatements                                        */
/* ------------------------------------------------------------------------- */

typedef struct {
  float min_x, max_x, min_y, max_y;
} env_t;

/* Sliding +-5 index envelope of each t1 trajectory (dtw.cpp:17-34,
 * lcss.cpp:15-35, frechet.cpp:16-33). */
static env_t* build_envelopes(const float* t1, int num_t, int n) {
  const int r = 5;
  env_t* envs = (env_t*)malloc(sizeof(env_t) * (size_t)num_t * n);
#pragma omp parallel for
  for (int t = 0; t < num_t; t++) {
    for (int i = 0; i < n; i++) {
      float min_x = F_BIG, max_x = -F_BIG, min_y = F_BIG, max_y = -F_BIG;
      int s = i - r > 0 ? i - r : 0;
      int e = i + r < n - 1 ? i + r : n - 1;
      for (int k = s; k <= e; k++) {
        float px = t1[2 * ((size_t)t * n + k)], py = t1[2 * ((size_t)t * n + k) + 1];
        min_x = smin(min_x, px);
        max_x = smax(max_x, px);
        min_y = smin(min_y, py);
        max_y = smax(max_y, py);
      }
      env_t ev = {min_x, max_x, min_y, max_y};
      envs[(size_t)t * n + i] = ev;
    }
  }
  return envs;
}

typedef struct {
  float key;
  int idx;
} kv_t;

/* Ascending (key, idx): the order std::partial_sort gives a
 * std::vector<std::pair<float,int>> (dtw.cpp:62, frechet.cpp:67). */
static int kv_cmp_asc(const void* a, const void* b) {
  const kv_t* x = (const kv_t*)a;
  const kv_t* y = (const kv_t*)b;
  if (x->key < y->key) return -1;
  if (x->key > y->key) return 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}
/* Descending key, then ascending index: std::stable_sort with a `>` key
 * comparator keeps equal keys in index order (lcss.cpp:67-70). */
static int kv_cmp_desc(const void* a, const void* b) {
  const kv_t* x = (const kv_t*)a;
  const kv_t* y = (const kv_t*)b;
  if (x->key > y->key) return -1;
  if (x->key < y->key) return 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}

/* Envelope-to-point distance term (dtw.cpp:54-56, frechet.cpp:55-57). */
static inline float env_point_dist(env_t e, float px, float py) {
  float dx = smax(0.0f, smax(e.min_x - px, px - e.max_x));
  float dy = smax(0.0f, smax(e.min_y - py, py - e.max_y));
  return sqrtf(dx * dx + dy * dy);
}

static inline float pdist(const float* p, const float* q) {
  float dx = p[0] - q[0];
  float dy = p[1] - q[1];
  return sqrtf(dx * dx + dy * dy);
}

/* CudaRuntime1/dtw.cpp:14-113 */
float orc_ref_dtw(const float* t1, const float* t2, float* out, int num_t, int n, int m) {
  double t0 = now_ms();
  env_t* envs = build_envelopes(t1, num_t, n);
  int K = num_t < 10 ? num_t : 10;
#pragma omp parallel
  {
    kv_t* lb = (kv_t*)malloc(sizeof(kv_t) * num_t);
    float* prev = (float*)malloc(sizeof(float) * (m + 1));
    float* curr = (float*)malloc(sizeof(float) * (m + 1));
#pragma omp for
    for (int i = 0; i < num_t; i++) {
      const env_t* ev = envs + (size_t)i * n;
      for (int j = 0; j < num_t; j++) {
        const float* c = t2 + 2 * (size_t)j * m;
        float s = 0.0f;
        for (int v = 0; v < m; v++) s += env_point_dist(ev[v * n / m], c[2 * v], c[2 * v + 1]);
        lb[j].key = s;
        lb[j].idx = j;
      }
      qsort(lb, num_t, sizeof(kv_t), kv_cmp_asc);
      float best = F_BIG;
      const float* a = t1 + 2 * (size_t)i * n;
      for (int k = 0; k < K; k++) {
        const float* b = t2 + 2 * (size_t)lb[k].idx * m;
        for (int v = 0; v <= m; v++) prev[v] = F_BIG;
        prev[0] = 0.0f;
        for (int u = 1; u <= n; u++) {
          curr[0] = F_BIG;
          for (int v = 1; v <= m; v++) {
            float cost = pdist(a + 2 * (u - 1), b + 2 * (v - 1));
            curr[v] = cost + smin(smin(prev[v], curr[v - 1]), prev[v - 1]);
          }
          float* t = prev;
          prev = curr;
          curr = t;
        }
        if (prev[m] < best) best = prev[m];
      }
      out[i] = best;
    }
    free(lb);
    free(prev);
    free(curr);
  }
  free(envs);
  return (float)(now_ms() - t0);
}

/* CudaRuntime1/lcss.cpp:13-115 */
float orc_ref_lcss(const float* t1, const float* t2, float* out, int num_t, int n, int m,
                   float epsilon) {
  double t0 = now_ms();
  env_t* envs = build_envelopes(t1, num_t, n);
  int K = num_t < 10 ? num_t : 10;
  int min_len = n < m ? n : m;
#pragma omp parallel
  {
    kv_t* ub = (kv_t*)malloc(sizeof(kv_t) * num_t);
    int* prev = (int*)malloc(sizeof(int) * (m + 1));
    int* curr = (int*)malloc(sizeof(int) * (m + 1));
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < num_t; i++) {
      const env_t* ev = envs + (size_t)i * n;
      for (int j = 0; j < num_t; j++) {
        const float* c = t2 + 2 * (size_t)j * m;
        int cnt = 0;
        for (int v = 0; v < m; v++) {
          /* floor((double)v*n/m) == v*n/m for non-negative ints (lcss.cpp:52) */
          env_t e = ev[(int)floor((double)v * (double)n / (double)m)];
          float px = c[2 * v], py = c[2 * v + 1];
          if (px > e.min_x - epsilon && px < e.max_x + epsilon && py > e.min_y - epsilon &&
              py < e.max_y + epsilon)
            cnt++;
        }
        ub[j].key = (float)cnt / min_len;
        ub[j].idx = j;
      }
      qsort(ub, num_t, sizeof(kv_t), kv_cmp_desc);
      float best = -1.0f;
      const float* a = t1 + 2 * (size_t)i * n;
      for (int k = 0; k < K; k++) {
        const float* b = t2 + 2 * (size_t)ub[k].idx * m;
        for (int v = 0; v <= m; v++) prev[v] = 0;
        for (int u = 1; u <= n; u++) {
          curr[0] = 0;
          for (int v = 1; v <= m; v++) {
            float dx = fabsf(a[2 * (u - 1)] - b[2 * (v - 1)]);
            float dy = fabsf(a[2 * (u - 1) + 1] - b[2 * (v - 1) + 1]);
            if (dx < epsilon && dy < epsilon)
              curr[v] = prev[v - 1] + 1;
            else
              curr[v] = prev[v] > curr[v - 1] ? prev[v] : curr[v - 1];
          }
          int* t = prev;
          prev = curr;
          curr = t;
        }
        float sim = (float)prev[m] / min_len;
        if (sim > best) best = sim;
      }
      out[i] = best;
    }
    free(ub);
    free(prev);
    free(curr);
  }
  free(envs);
  return (float)(now_ms() - t0);
}

/* CudaRuntime1/frechet.cpp:13-124 (rolling rows; same values as its full table) */
float orc_ref_frechet(const float* t1, const float* t2, float* out, int num_t, int n, int m) {
  double t0 = now_ms();
  env_t* envs = build_envelopes(t1, num_t, n);
  int K = num_t < 10 ? num_t : 10;
#pragma omp parallel
  {
    kv_t* lb = (kv_t*)malloc(sizeof(kv_t) * num_t);
    float* prev = (float*)malloc(sizeof(float) * (m + 1));
    float* curr = (float*)malloc(sizeof(float) * (m + 1));
#pragma omp for schedule(static)
    for (int i = 0; i < num_t; i++) {
      const env_t* ev = envs + (size_t)i * n;
      for (int j = 0; j < num_t; j++) {
        const float* c = t2 + 2 * (size_t)j * m;
        float s = 0.0f;
        for (int v = 0; v < m; v++) s = smax(s, env_point_dist(ev[v * n / m], c[2 * v], c[2 * v + 1]));
        lb[j].key = s;
        lb[j].idx = j;
      }
      qsort(lb, num_t, sizeof(kv_t), kv_cmp_asc);
      float best = F_BIG;
      const float* a = t1 + 2 * (size_t)i * n;
      for (int k = 0; k < K; k++) {
        const float* b = t2 + 2 * (size_t)lb[k].idx * m;
        /* row u = 1 (frechet.cpp:90, 98-100) */
        prev[1] = pdist(a, b);
        for (int v = 2; v <= m; v++) prev[v] = smax(prev[v - 1], pdist(a, b + 2 * (v - 1)));
        for (int u = 2; u <= n; u++) {
          curr[1] = smax(prev[1], pdist(a + 2 * (u - 1), b)); /* frechet.cpp:93-95 */
          for (int v = 2; v <= m; v++) {
            float d = pdist(a + 2 * (u - 1), b + 2 * (v - 1));
            float pm = smin(smin(prev[v], curr[v - 1]), prev[v - 1]);
            curr[v] = smax(d, pm);
          }
          float* t = prev;
          prev = curr;
          curr = t;
        }
        if (prev[m] < best) best = prev[m];
      }
      out[i] = best;
    }
    free(lb);
    free(prev);
    free(curr);
  }
  free(envs);
  return (float)(now_ms() - t0);
}

/* CudaRuntime1/hausdorff.cpp:11-109: uniform G x G grid over the target,
 * ring search around each source point, early break once a source point's
 * nearest distance cannot raise the running max. */
float orc_ref_directed_hausdorff_grid(const float* src, int len_src, const float* tgt,
                                      int len_tgt, float seed) {
  float min_x = tgt[0], max_x = tgt[0], min_y = tgt[1], max_y = tgt[1];
  for (int i = 1; i < len_tgt; i++) {
    min_x = smin(min_x, tgt[2 * i]);
    max_x = smax(max_x, tgt[2 * i]);
    min_y = smin(min_y, tgt[2 * i + 1]);
    max_y = smax(max_y, tgt[2 * i + 1]);
  }
  int G = (int)sqrt((double)len_tgt);
  if (G < 1) G = 1;
  float cw = (max_x - min_x) / G, ch = (max_y - min_y) / G;
  if (cw < 1e-6f) cw = 1e-6f;
  if (ch < 1e-6f) ch = 1e-6f;
  /* bucket target points by cell (counting sort keeps insertion order) */
  int* cell_of = (int*)malloc(sizeof(int) * len_tgt);
  int* start = (int*)calloc((size_t)G * G + 1, sizeof(int));
  int* items = (int*)malloc(sizeof(int) * len_tgt);
  for (int i = 0; i < len_tgt; i++) {
    int cx = (int)((tgt[2 * i] - min_x) / cw);
    int cy = (int)((tgt[2 * i + 1] - min_y) / ch);
    cx = cx < 0 ? 0 : (cx > G - 1 ? G - 1 : cx);
    cy = cy < 0 ? 0 : (cy > G - 1 ? G - 1 : cy);
    cell_of[i] = cy * G + cx;
    start[cell_of[i] + 1]++;
  }
  for (int c = 0; c < G * G; c++) start[c + 1] += start[c];
  int* fill = (int*)malloc(sizeof(int) * ((size_t)G * G));
  memcpy(fill, start, sizeof(int) * ((size_t)G * G));
  for (int i = 0; i < len_tgt; i++) items[fill[cell_of[i]]++] = i;

  float max_min = seed;
  for (int i = 0; i < len_src; i++) {
    float px = src[2 * i], py = src[2 * i + 1];
    float min_d2 = F_BIG;
    int cx0 = (int)((px - min_x) / cw);
    int cy0 = (int)((py - min_y) / ch);
    cx0 = cx0 < 0 ? 0 : (cx0 > G - 1 ? G - 1 : cx0);
    cy0 = cy0 < 0 ? 0 : (cy0 > G - 1 ? G - 1 : cy0);
    for (int r = 0; r <= G; r++) {
      int xa = cx0 - r, xb = cx0 + r, ya = cy0 - r, yb = cy0 + r;
      for (int cy = ya; cy <= yb; cy++) {
        for (int cx = xa; cx <= xb; cx++) {
          if (r > 0 && !(cy == ya || cy == yb || cx == xa || cx == xb)) continue;
          if (cx < 0 || cx >= G || cy < 0 || cy >= G) continue;
          float c_min_x = min_x + cx * cw, c_max_x = c_min_x + cw;
          float c_min_y = min_y + cy * ch, c_max_y = c_min_y + ch;
          float dxc = smax(smax(0.0f, c_min_x - px), px - c_max_x);
          float dyc = smax(smax(0.0f, c_min_y - py), py - c_max_y);
          if (dxc * dxc + dyc * dyc >= min_d2) continue;
          int cell = cy * G + cx;
          for (int it = start[cell]; it < start[cell + 1]; it++) {
            int t = items[it];
            float dx = px - tgt[2 * t], dy = py - tgt[2 * t + 1];
            float d2 = dx * dx + dy * dy;
            if (d2 < min_d2) min_d2 = d2;
            if (min_d2 <= max_min) goto early_prune;
          }
        }
      }
      {
        float bx0 = min_x + xa * cw, bx1 = min_x + (xb + 1) * cw;
        float by0 = min_y + ya * ch, by1 = min_y + (yb + 1) * ch;
        float dxb = smax(smax(0.0f, bx0 - px), px - bx1);
        float dyb = smax(smax(0.0f, by0 - py), py - by1);
        if (dxb * dxb + dyb * dyb >= min_d2) break;
      }
    }
  early_prune:
    if (min_d2 > max_min) max_min = min_d2;
  }
  free(cell_of);
  free(start);
  free(items);
  free(fill);
  return max_min;
}

void orc_ref_hausdorff_cands(const float* t1, int num_t1, int n, const float* t2, int num_t2,
                             int m, const int* cand, int top_k, float* out) {
  (void)num_t2;
#pragma omp parallel for
  for (int i = 0; i < num_t1; i++) {
    const float* A = t1 + 2 * (size_t)i * n;
    float best = F_BIG;
    for (int k = 0; k < top_k; k++) {
      const float* B = t2 + 2 * (size_t)cand[(size_t)i * top_k + k] * m;
      float d1 = orc_ref_directed_hausdorff_grid(A, n, B, m, 0.0f);
      float d2 = orc_ref_directed_hausdorff_grid(B, m, A, n, d1);
      if (d2 < best) best = d2;
    }
    out[i] = sqrtf(best);
  }
}

/* calc_exact_dist_sq, CudaRuntime1/euclidean.cpp:27-40 */
static double exact_dist_sq(const float* a, const float* b, int n, double cur_min) {
  double s = 0.0;
  for (int j = 0; j < n; j++) {
    double dx = (double)a[2 * j] - (double)b[2 * j];
    double dy = (double)a[2 * j + 1] - (double)b[2 * j + 1];
    s += dx * dx + dy * dy;
    if (s >= cur_min) return s;
  }
  return s;
}

void orc_ref_euclid_cands(const float* t1, const float* t2, const int* cand,
                          const int* offsets, float* out, int num_t, int n) {
#pragma omp parallel for
  for (int i = 0; i < num_t; i++) {
    double best = 1.7976931348623157e308;
    for (int e = offsets[i]; e < offsets[i + 1]; e++) {
      double s = exact_dist_sq(t1 + 2 * (size_t)i * n, t2 + 2 * (size_t)cand[e] * n, n, best);
      if (s < best) best = s;
    }
    out[i] = (float)sqrt(best);
  }
}

typedef struct {
  float x0, y0, x1, y1;
} box_t;

static box_t traj_box(const float* t, int len) {
  box_t b = {t[0], t[1], t[0], t[1]};
  for (int i = 1; i < len; i++) {
    b.x0 = smin(b.x0, t[2 * i]);
    b.x1 = smax(b.x1, t[2 * i]);
    b.y0 = smin(b.y0, t[2 * i + 1]);
    b.y1 = smax(b.y1, t[2 * i + 1]);
  }
  return b;
}

static inline float box_box_d2(box_t a, box_t b) {
  float dx = smax(0.0f, smax(a.x0 - b.x1, b.x0 - a.x1));
  float dy = smax(0.0f, smax(a.y0 - b.y1, b.y0 - a.y1));
  return dx * dx + dy * dy;
}

void orc_mbr_knn(const float* t1, int num_t1, int n, const float* t2, int num_t2, int m, int k,
                 int* out) {
  box_t* boxes = (box_t*)malloc(sizeof(box_t) * (num_t2 > 0 ? num_t2 : 1));
  for (int j = 0; j < num_t2; j++) boxes[j] = traj_box(t2 + 2 * (size_t)j * m, m);
#pragma omp parallel
  {
    kv_t* kv = (kv_t*)malloc(sizeof(kv_t) * (num_t2 > 0 ? num_t2 : 1));
#pragma omp for
    for (int i = 0; i < num_t1; i++) {
      box_t q = traj_box(t1 + 2 * (size_t)i * n, n);
      for (int j = 0; j < num_t2; j++) {
        kv[j].key = box_box_d2(q, boxes[j]);
        kv[j].idx = j;
      }
      qsort(kv, num_t2, sizeof(kv_t), kv_cmp_asc);
      int got = num_t2 < k ? num_t2 : k;
      for (int e = 0; e < got; e++) out[(size_t)i * k + e] = kv[e].idx;
      for (int e = got; e < k; e++) out[(size_t)i * k + e] = got > 0 ? kv[got - 1].idx : 0;
    }
    free(kv);
  }
  free(boxes);
}

/* ------------------------------------------------------------------------- */
/* 2. FP64 exact measures                                                     */
/* ------------------------------------------------------------------------- */

static inline double d2_64(const float* p, const float* q) {
  double dx = (double)p[0] - (double)q[0];
  double dy = (double)p[1] - (double)q[1];
  return dx * dx + dy * dy;
}

/* Banded DTW, D(i,j) = cost(i,j) + min(D(i-1,j), D(i,j-1), D(i-1,j-1)),
 * D(-1,-1) = 0, cells outside the band = +inf.  Early abandon when every
 * cell of a row exceeds `abandon` (a warping path visits every row and D
 * never decreases along it). */
static double dtw64_core(const float* a, int n, const float* b, int m, int w, int cost,
                         double abandon, double* prev, double* cur, int64_t* cells) {
  const double INF = INFINITY;
  int plo = 0, phi = -1; /* previous row's band; row -1 holds only D(-1,-1)=0 */
  for (int i = 0; i < n; i++) {
    int lo, hi;
    orc_band_row(i, n, m, w, &lo, &hi);
    if (lo > hi) return INF;
    double rowmin = INF;
    const float* ai = a + 2 * i;
    for (int j = lo; j <= hi; j++) {
      double up, dg, lf;
      if (i == 0) {
        up = INF;
        dg = (j == 0) ? 0.0 : INF;
      } else {
        up = (j >= plo && j <= phi) ? prev[j] : INF;
        dg = (j - 1 >= plo && j - 1 <= phi) ? prev[j - 1] : INF;
      }
      lf = (j - 1 >= lo) ? cur[j - 1] : INF;
      double mn = up < lf ? up : lf;
      mn = dg < mn ? dg : mn;
      double c = d2_64(ai, b + 2 * j);
      if (cost == ORC_COST_EUCLID) c = sqrt(c);
      double v = c + mn;
      cur[j] = v;
      if (v < rowmin) rowmin = v;
    }
    if (cells) *cells += hi - lo + 1;
    if (rowmin > abandon) return INF;
    double* t = prev;
    prev = cur;
    cur = t;
    plo = lo;
    phi = hi;
  }
  /* after the final swap the last row lives in prev */
  return (m - 1 >= plo && m - 1 <= phi) ? prev[m - 1] : INF;
}

double orc_dtw64(const float* a, int n, const float* b, int m, int band_pct, int cost) {
  double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)m);
  int w = orc_band_w(n, m, band_pct);
  double r = dtw64_core(a, n, b, m, w, cost, INFINITY, buf, buf + m, NULL);
  free(buf);
  return r;
}

int orc_lcss_count(const float* a, int n, const float* b, int m, float eps, int delta) {
  int* prev = (int*)calloc((size_t)m + 1, sizeof(int));
  int* cur = (int*)calloc((size_t)m + 1, sizeof(int));
  for (int u = 1; u <= n; u++) {
    cur[0] = 0;
    for (int v = 1; v <= m; v++) {
      int inwin = delta < 0 || abs(u - v) <= delta;
      float dx = fabsf(a[2 * (u - 1)] - b[2 * (v - 1)]);
      float dy = fabsf(a[2 * (u - 1) + 1] - b[2 * (v - 1) + 1]);
      if (inwin && dx < eps && dy < eps)
        cur[v] = prev[v - 1] + 1;
      else
        cur[v] = prev[v] > cur[v - 1] ? prev[v] : cur[v - 1];
    }
    int* t = prev;
    prev = cur;
    cur = t;
  }
  int r = prev[m];
  free(prev);
  free(cur);
  return r;
}

/* Discrete Frechet in the squared domain, sqrt at the end (sqrt is monotone
 * and correctly rounded, so it commutes with the max/min recursion). */
double orc_frechet64(const float* a, int n, const float* b, int m) {
  const double INF = INFINITY;
  double* prev = (double*)malloc(sizeof(double) * m);
  double* cur = (double*)malloc(sizeof(double) * m);
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < m; j++) {
      double d = d2_64(a + 2 * i, b + 2 * j);
      double mn;
      if (i == 0 && j == 0)
        mn = 0.0;
      else {
        double up = i > 0 ? prev[j] : INF;
        double lf = j > 0 ? cur[j - 1] : INF;
        double dg = (i > 0 && j > 0) ? prev[j - 1] : INF;
        mn = up < lf ? up : lf;
        mn = dg < mn ? dg : mn;
      }
      cur[j] = d > mn ? d : mn;
    }
    double* t = prev;
    prev = cur;
    cur = t;
  }
  double r = sqrt(prev[m - 1]);
  free(prev);
  free(cur);
  return r;
}

static double directed64(const float* A, int na, const float* B, int nb) {
  double mx = 0.0;
  for (int i = 0; i < na; i++) {
    double mn = INFINITY;
    for (int j = 0; j < nb; j++) {
      double d = d2_64(A + 2 * i, B + 2 * j);
      if (d < mn) mn = d;
    }
    if (mn > mx) mx = mn;
  }
  return mx;
}

double orc_hausdorff64(const float* a, int n, const float* b, int m) {
  double h1 = directed64(a, n, b, m), h2 = directed64(b, m, a, n);
  return sqrt(h1 > h2 ? h1 : h2);
}

double orc_euclid64(const float* q, int n, const float* c, int m) {
  if (n < m) return INFINITY;
  double s = 0.0;
  for (int i = 0; i < m; i++) s += d2_64(q + 2 * i, c + 2 * i);
  return sqrt(s);
}

/* ------------------------------------------------------------------------- */
/* brute-force kNN                                                            */
/* ------------------------------------------------------------------------- */

typedef struct {
  double key;
  int idx;
} dk_t;

static int dk_cmp(const void* a, const void* b) {
  const dk_t* x = (const dk_t*)a;
  const dk_t* y = (const dk_t*)b;
  if (x->key < y->key) return -1;
  if (x->key > y->key) return 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}

int orc_knn(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
            const float* dbpts, const int64_t* dboff, int ndb, int* ids, double* dists,
            int nthreads) {
  if (p->k <= 0) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
  {
    dk_t* kv = (dk_t*)malloc(sizeof(dk_t) * (ndb > 0 ? ndb : 1));
#pragma omp for schedule(dynamic, 1)
    for (int q = 0; q < nq; q++) {
      const float* a = qpts + 2 * qoff[q];
      int n = (int)(qoff[q + 1] - qoff[q]);
      for (int c = 0; c < ndb; c++) {
        const float* b = dbpts + 2 * dboff[c];
        int m = (int)(dboff[c + 1] - dboff[c]);
        double v;
        switch (p->measure) {
          case ORC_DTW: v = orc_dtw64(a, n, b, m, p->band_pct, p->cost); break;
          case ORC_LCSS: v = -(double)orc_lcss_count(a, n, b, m, p->epsilon, p->delta); break;
          case ORC_FRECHET: v = orc_frechet64(a, n, b, m); break;
          case ORC_HAUSDORFF: v = orc_hausdorff64(a, n, b, m); break;
          default: v = orc_euclid64(a, n, b, m); break;
        }
        kv[c].key = v;
        kv[c].idx = c;
      }
      qsort(kv, ndb, sizeof(dk_t), dk_cmp);
      for (int e = 0; e < p->k; e++) {
        if (e < ndb) {
          ids[(size_t)q * p->k + e] = kv[e].idx;
          dists[(size_t)q * p->k + e] = p->measure == ORC_LCSS ? -kv[e].key : kv[e].key;
        } else {
          ids[(size_t)q * p->k + e] = -1;
          dists[(size_t)q * p->k + e] = p->measure == ORC_LCSS ? -1.0 : INFINITY;
        }
      }
    }
    free(kv);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* pruned exact DTW kNN (CPU baseline)                                        */
/* ------------------------------------------------------------------------- */

typedef struct {
  int levels, n;
  float* mn_x; /* [levels][n] */
  float* mx_x;
  float* mn_y;
  float* mx_y;
} sparse_t;

static void sparse_build(sparse_t* s, const float* a, int n) {
  int L = 1;
  while ((1 << L) <= n) L++;
  s->levels = L;
  s->n = n;
  s->mn_x = (float*)malloc(sizeof(float) * (size_t)L * n * 4);
  s->mx_x = s->mn_x + (size_t)L * n;
  s->mn_y = s->mx_x + (size_t)L * n;
  s->mx_y = s->mn_y + (size_t)L * n;
  for (int i = 0; i < n; i++) {
    s->mn_x[i] = s->mx_x[i] = a[2 * i];
    s->mn_y[i] = s->mx_y[i] = a[2 * i + 1];
  }
  for (int l = 1; l < L; l++) {
    int h = 1 << (l - 1);
    for (int i = 0; i + (1 << l) <= n; i++) {
      size_t o = (size_t)l * n + i, p0 = (size_t)(l - 1) * n + i, p1 = p0 + h;
      s->mn_x[o] = fminf(s->mn_x[p0], s->mn_x[p1]);
      s->mx_x[o] = fmaxf(s->mx_x[p0], s->mx_x[p1]);
      s->mn_y[o] = fminf(s->mn_y[p0], s->mn_y[p1]);
      s->mx_y[o] = fmaxf(s->mx_y[p0], s->mx_y[p1]);
    }
  }
}

/* squared distance from point c to the bounding box of a[lo..hi] */
static inline double sparse_box_d2(const sparse_t* s, int lo, int hi, const float* c) {
  int len = hi - lo + 1, l = 0;
  while ((2 << l) <= len) l++;
  size_t o0 = (size_t)l * s->n + lo, o1 = (size_t)l * s->n + hi - (1 << l) + 1;
  double x0 = fminf(s->mn_x[o0], s->mn_x[o1]), x1 = fmaxf(s->mx_x[o0], s->mx_x[o1]);
  double y0 = fminf(s->mn_y[o0], s->mn_y[o1]), y1 = fmaxf(s->mx_y[o0], s->mx_y[o1]);
  double cx = c[0], cy = c[1];
  double dx = cx < x0 ? x0 - cx : (cx > x1 ? cx - x1 : 0.0);
  double dy = cy < y0 ? y0 - cy : (cy > y1 ? cy - y1 : 0.0);
  return dx * dx + dy * dy;
}

typedef struct {
  double lb;
  int idx;
} lbk_t;

static int lbk_cmp(const void* a, const void* b) {
  const lbk_t* x = (const lbk_t*)a;
  const lbk_t* y = (const lbk_t*)b;
  if (x->lb < y->lb) return -1;
  if (x->lb > y->lb) return 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}

/* insert (v, idx) into an ascending (key, idx) list of capacity k */
static void topk_insert(dk_t* top, int* cnt, int k, double v, int idx) {
  if (*cnt == k) {
    dk_t* last = &top[k - 1];
    if (v > last->key || (v == last->key && idx > last->idx)) return;
    (*cnt)--;
  }
  int p = *cnt;
  while (p > 0 && (top[p - 1].key > v || (top[p - 1].key == v && top[p - 1].idx > idx))) {
    top[p] = top[p - 1];
    p--;
  }
  top[p].key = v;
  top[p].idx = idx;
  (*cnt)++;
}

int orc_dtw_knn_pruned(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
                       const float* dbpts, const int64_t* dboff, int ndb, int* ids,
                       double* dists, int nthreads, int64_t* cells_out) {
  int k = p->k;
  int64_t cells_total = 0;
  int maxm = 1;
  for (int c = 0; c < ndb; c++) {
    int m = (int)(dboff[c + 1] - dboff[c]);
    if (m > maxm) maxm = m;
  }
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
  /* margin covering FP64 rounding of bound versus DP (both ~1e-16 relative) */
  const double slack = 1.0 + 1e-12;
#pragma omp parallel num_threads(nthreads) reduction(+ : cells_total)
  {
    lbk_t* order = (lbk_t*)malloc(sizeof(lbk_t) * (ndb > 0 ? ndb : 1));
    double* rows = (double*)malloc(sizeof(double) * 2 * (size_t)maxm);
    dk_t* top = (dk_t*)malloc(sizeof(dk_t) * k);
#pragma omp for schedule(dynamic, 1)
    for (int q = 0; q < nq; q++) {
      const float* a = qpts + 2 * qoff[q];
      int n = (int)(qoff[q + 1] - qoff[q]);
      sparse_t sp;
      sparse_build(&sp, a, n);
      for (int c = 0; c < ndb; c++) {
        const float* b = dbpts + 2 * dboff[c];
        int m = (int)(dboff[c + 1] - dboff[c]);
        int w = orc_band_w(n, m, p->band_pct);
        double lb = 0.0;
        int feasible = 1;
        for (int j = 0; j < m; j++) {
          int lo, hi;
          orc_band_row(j, m, n, w, &lo, &hi); /* rows of column j */
          if (lo > hi) {
            feasible = 0;
            break;
          }
          double t;
          if (j == 0)
            t = d2_64(a, b);
          else if (j == m - 1)
            t = d2_64(a + 2 * (n - 1), b + 2 * j);
          else
            t = sparse_box_d2(&sp, lo, hi, b + 2 * j);
          if (p->cost == ORC_COST_EUCLID) t = sqrt(t);
          lb += t;
        }
        if (m == 1 && n > 1) {
          double t = d2_64(a + 2 * (n - 1), b);
          lb += p->cost == ORC_COST_EUCLID ? sqrt(t) : t;
        }
        order[c].lb = feasible ? lb : INFINITY;
        order[c].idx = c;
      }
      free(sp.mn_x);
      qsort(order, ndb, sizeof(lbk_t), lbk_cmp);
      int cnt = 0;
      double thr = INFINITY;
      for (int e = 0; e < ndb; e++) {
        if (order[e].lb > thr || order[e].lb == INFINITY) break;
        int c = order[e].idx;
        const float* b = dbpts + 2 * dboff[c];
        int m = (int)(dboff[c + 1] - dboff[c]);
        int w = orc_band_w(n, m, p->band_pct);
        int64_t cells = 0;
        double v = dtw64_core(a, n, b, m, w, p->cost, thr, rows, rows + maxm, &cells);
        cells_total += cells;
        if (v != INFINITY) topk_insert(top, &cnt, k, v, c);
        if (cnt == k) thr = top[k - 1].key * slack;
      }
      for (int e = 0; e < k; e++) {
        ids[(size_t)q * k + e] = e < cnt ? top[e].idx : -1;
        dists[(size_t)q * k + e] = e < cnt ? top[e].key : INFINITY;
      }
    }
    free(order);
    free(rows);
    free(top);
  }
  if (cells_out) *cells_out = cells_total;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* pruned exact kNN for every measure (parity checks on large databases)      */
/* ------------------------------------------------------------------------- */

/* Every bound below is a valid bound on the key the brute force ranks by,
 * as computed in FP64: the rounding of each operation is monotone, so a
 * bound assembled from the same float coordinates by the same (or fewer,
 * smaller) operations never exceeds the computed value.  Candidates are
 * visited in bound order in parallel chunks; a chunk is evaluated against
 * the k-th key known when it starts (early abandon only when the computed
 * value already exceeds it), and the visit stops at the first bound above
 * the k-th key.  The result equals orc_knn's, ties included. */

typedef struct {
  double x0, x1, y0, y1;
} dbox_t;

static dbox_t box64(const float* t, int len) {
  dbox_t b = {t[0], t[0], t[1], t[1]};
  for (int i = 1; i < len; i++) {
    double x = t[2 * i], y = t[2 * i + 1];
    if (x < b.x0) b.x0 = x;
    if (x > b.x1) b.x1 = x;
    if (y < b.y0) b.y0 = y;
    if (y > b.y1) b.y1 = y;
  }
  return b;
}

/* squared distance from p to the box: each axis gap is the difference of p
 * and the nearest box edge, itself a coordinate of some point, so it never
 * exceeds the computed gap to any point of the box's trajectory */
static inline double ptbox_d2(const float* p, dbox_t b) {
  double px = p[0], py = p[1];
  double dx = px < b.x0 ? b.x0 - px : (px > b.x1 ? px - b.x1 : 0.0);
  double dy = py < b.y0 ? b.y0 - py : (py > b.y1 ? py - b.y1 : 0.0);
  return dx * dx + dy * dy;
}

/* max over the points of t of their squared distance to box b */
static double max_ptbox_d2(const float* t, int len, dbox_t b) {
  double mx = 0.0;
  for (int i = 0; i < len; i++) {
    double d = ptbox_d2(t + 2 * i, b);
    if (d > mx) mx = d;
  }
  return mx;
}

/* LCSS: points of t that could match some point of the set boxed by b
 * (|dx| < eps and |dy| < eps in float, as orc_lcss_count tests them) */
static int lcss_matchable(const float* t, int len, const float* bx, int blen, float eps) {
  float x0 = bx[0], x1 = bx[0], y0 = bx[1], y1 = bx[1];
  for (int j = 1; j < blen; j++) {
    float x = bx[2 * j], y = bx[2 * j + 1];
    if (x < x0) x0 = x;
    if (x > x1) x1 = x;
    if (y < y0) y0 = y;
    if (y > y1) y1 = y;
  }
  int cnt = 0;
  for (int i = 0; i < len; i++) {
    float x = t[2 * i], y = t[2 * i + 1];
    int out = (x > x1 && fabsf(x - x1) >= eps) || (x < x0 && fabsf(x - x0) >= eps) ||
              (y > y1 && fabsf(y - y1) >= eps) || (y < y0 && fabsf(y - y0) >= eps);
    cnt += !out;
  }
  return cnt;
}

/* discrete Frechet (orc_frechet64's arithmetic) abandoning once a row's
 * smallest value has a square root above thr */
static double frechet64_ab(const float* a, int n, const float* b, int m, double thr) {
  const double INF = INFINITY;
  double* prev = (double*)malloc(sizeof(double) * 2 * (size_t)m);
  double* cur = prev + m;
  double r = INF;
  for (int i = 0; i < n; i++) {
    double rowmin = INF;
    for (int j = 0; j < m; j++) {
      double d = d2_64(a + 2 * i, b + 2 * j);
      double mn;
      if (i == 0 && j == 0)
        mn = 0.0;
      else {
        double up = i > 0 ? prev[j] : INF;
        double lf = j > 0 ? cur[j - 1] : INF;
        double dg = (i > 0 && j > 0) ? prev[j - 1] : INF;
        mn = up < lf ? up : lf;
        mn = dg < mn ? dg : mn;
      }
      cur[j] = d > mn ? d : mn;
      if (cur[j] < rowmin) rowmin = cur[j];
    }
    if (sqrt(rowmin) > thr) goto done;
    double* t = prev;
    prev = cur;
    cur = t;
  }
  r = sqrt(prev[m - 1]);
done:
  free(prev < cur ? prev : cur);
  return r;
}

/* directed64 with the early break of a point whose running minimum cannot
 * raise the maximum, abandoning once the maximum's root exceeds thr;
 * returns the squared directed distance, or +inf when abandoned */
static double directed64_ab(const float* A, int na, const float* B, int nb, double mx,
                            double thr) {
  for (int i = 0; i < na; i++) {
    double mn = INFINITY;
    for (int j = 0; j < nb; j++) {
      double d = d2_64(A + 2 * i, B + 2 * j);
      if (d < mn) {
        mn = d;
        if (mn <= mx) break;
      }
    }
    if (mn > mx) {
      mx = mn;
      if (sqrt(mx) > thr) return INFINITY;
    }
  }
  return mx;
}

static double euclid64_ab(const float* q, int n, const float* c, int m, double thr) {
  if (n < m) return INFINITY;
  double s = 0.0;
  for (int i = 0; i < m; i++) {
    s += d2_64(q + 2 * i, c + 2 * i);
    if ((i & 15) == 15 && sqrt(s) > thr) return INFINITY;
  }
  return sqrt(s);
}

/* banded LB_Keogh of DTW over the candidate's columns (first and last
 * columns exact), as the CPU baseline computes it */
static double dtw_lb64(const orc_params* p, const sparse_t* sp, const float* a, int n,
                       const float* b, int m) {
  int w = orc_band_w(n, m, p->band_pct);
  double lb = 0.0;
  for (int j = 0; j < m; j++) {
    int lo, hi;
    orc_band_row(j, m, n, w, &lo, &hi);
    if (lo > hi) return INFINITY;
    double t;
    if (j == 0)
      t = d2_64(a, b);
    else if (j == m - 1)
      t = d2_64(a + 2 * (n - 1), b + 2 * j);
    else
      t = sparse_box_d2(sp, lo, hi, b + 2 * j);
    if (p->cost == ORC_COST_EUCLID) t = sqrt(t);
    lb += t;
  }
  if (m == 1 && n > 1) {
    double t = d2_64(a + 2 * (n - 1), b);
    lb += p->cost == ORC_COST_EUCLID ? sqrt(t) : t;
  }
  return lb;
}

int orc_knn_pruned(const orc_params* p, const float* qpts, const int64_t* qoff, int nq,
                   const float* dbpts, const int64_t* dboff, int ndb, int* ids, double* dists,
                   int nthreads, int64_t* evaluated_out) {
  const int k = p->k;
  if (k <= 0) return 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
  const int lcss = p->measure == ORC_LCSS;
  /* DTW's bound and DP sum round differently (both ~1e-16 relative) */
  const double slack = p->measure == ORC_DTW ? 1.0 + 1e-12 : 1.0;
  int maxm = 1;
  for (int c = 0; c < ndb; c++) {
    int m = (int)(dboff[c + 1] - dboff[c]);
    if (m > maxm) maxm = m;
  }
  lbk_t* order = (lbk_t*)malloc(sizeof(lbk_t) * (ndb > 0 ? ndb : 1));
  int chunk_cap = 8 * nthreads;
  double* val = (double*)malloc(sizeof(double) * chunk_cap);
  dk_t* top = (dk_t*)malloc(sizeof(dk_t) * k);
  int64_t evaluated = 0;
  for (int q = 0; q < nq; q++) {
    const float* a = qpts + 2 * qoff[q];
    const int n = (int)(qoff[q + 1] - qoff[q]);
    const dbox_t qb = box64(a, n);
    sparse_t sp;
    sp.mn_x = NULL;
    if (p->measure == ORC_DTW) sparse_build(&sp, a, n);
    /* keys: the brute force's ranking key (LCSS: minus the count) */
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int c = 0; c < ndb; c++) {
      const float* b = dbpts + 2 * dboff[c];
      const int m = (int)(dboff[c + 1] - dboff[c]);
      double lb;
      switch (p->measure) {
        case ORC_DTW: lb = dtw_lb64(p, &sp, a, n, b, m); break;
        case ORC_LCSS: {
          int ua = lcss_matchable(a, n, b, m, p->epsilon);
          int ub = lcss_matchable(b, m, a, n, p->epsilon);
          lb = -(double)(ua < ub ? ua : ub);
          break;
        }
        case ORC_FRECHET:
        case ORC_HAUSDORFF: {
          double e2 = max_ptbox_d2(b, m, qb), d2 = max_ptbox_d2(a, n, box64(b, m));
          if (p->measure == ORC_FRECHET) {
            double t = d2_64(a, b);
            if (t > e2) e2 = t;
            t = d2_64(a + 2 * (n - 1), b + 2 * (m - 1));
            if (t > e2) e2 = t;
          }
          lb = sqrt(e2 > d2 ? e2 : d2);
          break;
        }
        default: { /* lock-step: the first and last terms of the sum */
          if (n < m) {
            lb = INFINITY;
          } else {
            double s = d2_64(a, b);
            if (m > 1) s += d2_64(a + 2 * (m - 1), b + 2 * (m - 1));
            lb = sqrt(s);
          }
          break;
        }
      }
      order[c].lb = lb;
      order[c].idx = c;
    }
    free(sp.mn_x);
    qsort(order, ndb, sizeof(lbk_t), lbk_cmp);
    int cnt = 0;
    double thr = INFINITY;
    int e = 0;
    while (e < ndb) {
      if (cnt == k && order[e].lb > thr * slack) break;
      int nch = 0;
      while (nch < chunk_cap && e + nch < ndb && !(cnt == k && order[e + nch].lb > thr * slack))
        nch++;
      const double thr0 = thr;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
      for (int t = 0; t < nch; t++) {
        const int c = order[e + t].idx;
        const float* b = dbpts + 2 * dboff[c];
        const int m = (int)(dboff[c + 1] - dboff[c]);
        double v;
        switch (p->measure) {
          case ORC_DTW: {
            double* rows = (double*)malloc(sizeof(double) * 2 * (size_t)maxm);
            v = dtw64_core(a, n, b, m, orc_band_w(n, m, p->band_pct), p->cost, thr0, rows,
                           rows + maxm, NULL);
            free(rows);
            break;
          }
          case ORC_LCSS: v = -(double)orc_lcss_count(a, n, b, m, p->epsilon, p->delta); break;
          case ORC_FRECHET: v = frechet64_ab(a, n, b, m, thr0); break;
          case ORC_HAUSDORFF: {
            double h1 = directed64_ab(a, n, b, m, 0.0, thr0);
            double h = h1 == INFINITY ? INFINITY : directed64_ab(b, m, a, n, h1, thr0);
            v = h == INFINITY ? INFINITY : sqrt(h);
            break;
          }
          default: v = euclid64_ab(a, n, b, m, thr0); break;
        }
        val[t] = v;
      }
      evaluated += nch;
      /* abandoned values (+inf) lie above the k-th key and are refused */
      for (int t = 0; t < nch; t++) topk_insert(top, &cnt, k, val[t], order[e + t].idx);
      if (cnt == k) thr = top[k - 1].key;
      e += nch;
    }
    for (int x = 0; x < k; x++) {
      ids[(size_t)q * k + x] = x < cnt ? top[x].idx : -1;
      dists[(size_t)q * k + x] = x < cnt ? (lcss ? -top[x].key : top[x].key)
                                         : (lcss ? -1.0 : INFINITY);
    }
  }
  free(order);
  free(val);
  free(top);
  if (evaluated_out) *evaluated_out = evaluated;
  return 0;
}
