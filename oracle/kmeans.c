/*
 * Oracle restatement of smartcore's KMeans path (fit, k-means++ seeding, the
 * BBD-tree filtering step and predict).  TEST INFRASTRUCTURE ONLY (see
 * oracle.h).  Compiled with -ffp-contract=off: every sum below is evaluated
 * left to right, one rounding per operation, as rustc emits it.
 */
#define _POSIX_C_SOURCE 199309L
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static char g_err[256];
const char *orc_last_error(void) { return g_err; }

/* ---- element access: DenseMatrix::get (src/linalg/basic/matrix.rs:367-381) ---- */
typedef struct {
  int dtype, layout;
  const void *p;
  int64_t n, d, ld;
} mat;

static inline int64_t off(const mat *m, int64_t i, int64_t j) {
  return m->layout == ORC_ROW_MAJOR ? i * m->ld + j : j * m->ld + i;
}
static inline double getd(const mat *m, int64_t i, int64_t j) { /* to_f64(): exact */
  return m->dtype == ORC_F32 ? (double)((const float *)m->p)[off(m, i, j)]
                             : ((const double *)m->p)[off(m, i, j)];
}
static inline float getf(const mat *m, int64_t i, int64_t j) {
  return ((const float *)m->p)[off(m, i, j)];
}

/* Euclidian::squared_distance (src/metrics/distance/euclidian.rs:51-67):
 * per term r = a - b and r * r in the element type T, widened to f64, summed
 * in f64 from the first term to the last. */
static double sqd_f64(const double *a, const double *b, int64_t d) {
  double s = 0.0;
  for (int64_t j = 0; j < d; ++j) {
    double r = a[j] - b[j];
    s += r * r;
  }
  return s;
}
static double sqd_f32(const float *a, const float *b, int64_t d) {
  double s = 0.0;
  for (int64_t j = 0; j < d; ++j) {
    float r = a[j] - b[j];
    float rr = r * r;
    s += (double)rr;
  }
  return s;
}

double orc_sqdist(int dtype, const void *a, const void *b, int64_t d) {
  return dtype == ORC_F32 ? sqd_f32((const float *)a, (const float *)b, d)
                          : sqd_f64((const double *)a, (const double *)b, d);
}

/* ---- KMeans::kmeans_plus_plus (src/cluster/kmeans.rs:354-413) ---- */
/* The draws are passed in (first = gen_range(0..n), u[j-1] = gen::<f64>()),
 * so this function is independent of the generator. */
void orc_kmeanspp(int dtype, int layout, const void *x, int64_t n, int64_t d,
                  int64_t ld, int64_t k, int64_t first_index,
                  const double *uniforms, int64_t *y, int64_t *chosen) {
  mat m = {dtype, layout, x, n, d, ld};
  size_t es = dtype == ORC_F32 ? sizeof(float) : sizeof(double);
  char *row = malloc((size_t)d * es + 1), *cen = malloc((size_t)d * es + 1);
  double *dd = malloc((size_t)n * sizeof(double) + 1);
  int64_t ci = first_index;
  if (chosen) chosen[0] = ci;
#define LOADROW(dst, i)                                                     \
  for (int64_t j = 0; j < d; ++j) {                                         \
    if (dtype == ORC_F32) ((float *)(dst))[j] = getf(&m, (i), j);           \
    else ((double *)(dst))[j] = getd(&m, (i), j);                           \
  }
  LOADROW(cen, ci);
  for (int64_t i = 0; i < n; ++i) { y[i] = 0; dd[i] = DBL_MAX; }
  for (int64_t j = 1; j < k; ++j) {
    for (int64_t i = 0; i < n; ++i) { /* :368-379 */
      LOADROW(row, i);
      double dist = orc_sqdist(dtype, row, cen, d);
      if (dist < dd[i]) { dd[i] = dist; y[i] = j - 1; }
    }
    double sum = 0.0; /* :381-384 */
    for (int64_t i = 0; i < n; ++i) sum += dd[i];
    double cutoff = uniforms[j - 1] * sum; /* :385 */
    double cost = 0.0;
    int64_t index = 0;
    while (index < n) { /* :386-394 */
      cost += dd[index];
      if (cost >= cutoff) break;
      ++index;
    }
    ci = index; /* index == n would panic in the reference; it cannot be reached
                   because the last prefix equals sum >= cutoff */
    if (ci >= n) ci = n - 1;
    if (chosen) chosen[j] = ci;
    LOADROW(cen, ci);
  }
  for (int64_t i = 0; i < n; ++i) { /* :399-410 */
    LOADROW(row, i);
    double dist = orc_sqdist(dtype, row, cen, d);
    if (dist < dd[i]) { dd[i] = dist; y[i] = k - 1; }
  }
#undef LOADROW
  free(row); free(cen); free(dd);
}

/* ---- BBDTree (src/algorithm/neighbour/bbd_tree.rs) ---- */
typedef struct {
  int64_t count, index, lower, upper; /* lower/upper = -1 for a leaf */
  double cost;
} node;

typedef struct {
  int64_t d, nn, cap;
  node *nodes;
  double *center, *radius, *sum; /* nn x d each */
  int64_t *index;
  int64_t root;
} tree;

static int64_t add_node(tree *t) {
  if (t->nn == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 64;
    t->nodes = realloc(t->nodes, (size_t)t->cap * sizeof(node));
    t->center = realloc(t->center, (size_t)(t->cap * t->d) * sizeof(double));
    t->radius = realloc(t->radius, (size_t)(t->cap * t->d) * sizeof(double));
    t->sum = realloc(t->sum, (size_t)(t->cap * t->d) * sizeof(double));
  }
  return t->nn++;
}

/* node_cost (bbd_tree.rs:297-305) */
static double node_cost(const tree *t, int64_t nd, const double *c) {
  const node *q = &t->nodes[nd];
  const double *s = t->sum + nd * t->d;
  double scatter = 0.0;
  for (int64_t i = 0; i < t->d; ++i) {
    double v = (s[i] / (double)q->count) - c[i];
    scatter += v * v;
  }
  return q->cost + (double)q->count * scatter;
}

/* build_node (bbd_tree.rs:195-295).  Children are created before the parent
 * is stored, as in the reference, so a node's slot is assigned last. */
static int64_t build_node(tree *t, const mat *m, int64_t begin, int64_t end) {
  int64_t d = t->d;
  double *lb = malloc((size_t)d * sizeof(double)), *ub = malloc((size_t)d * sizeof(double));
  double *center = malloc((size_t)d * sizeof(double)), *radius = malloc((size_t)d * sizeof(double));
  double *sum = calloc((size_t)d, sizeof(double));
  node q = {end - begin, begin, -1, -1, 0.0};
  for (int64_t i = 0; i < d; ++i) lb[i] = ub[i] = getd(m, t->index[begin], i);
  for (int64_t i = begin; i < end; ++i)
    for (int64_t j = 0; j < d; ++j) {
      double c = getd(m, t->index[i], j);
      if (lb[j] > c) lb[j] = c;
      if (ub[j] < c) ub[j] = c;
    }
  double max_radius = -1.0;
  int64_t split = 0;
  for (int64_t i = 0; i < d; ++i) {
    center[i] = (lb[i] + ub[i]) / 2.0;
    radius[i] = (ub[i] - lb[i]) / 2.0;
    if (radius[i] > max_radius) { max_radius = radius[i]; split = i; }
  }
  if (max_radius < 1e-10) { /* leaf: one distinct point, possibly repeated */
    for (int64_t i = 0; i < d; ++i) sum[i] = getd(m, t->index[begin], i);
    if (end > begin + 1) {
      int64_t len = end - begin;
      for (int64_t i = 0; i < d; ++i) sum[i] *= (double)len;
    }
    q.cost = 0.0;
  } else {
    double cut = center[split];
    int64_t i1 = begin, i2 = end - 1, size = 0;
    while (i1 <= i2) {
      int g1 = getd(m, t->index[i1], split) < cut;
      int g2 = getd(m, t->index[i2], split) >= cut;
      if (!g1 && !g2) {
        int64_t tmp = t->index[i1]; t->index[i1] = t->index[i2]; t->index[i2] = tmp;
        g1 = g2 = 1;
      }
      if (g1) { ++i1; ++size; }
      if (g2) { --i2; }
    }
    q.lower = build_node(t, m, begin, begin + size);
    q.upper = build_node(t, m, begin + size, end);
    const double *sl = t->sum + q.lower * d, *su = t->sum + q.upper * d;
    for (int64_t i = 0; i < d; ++i) sum[i] = sl[i] + su[i];
    double *mean = malloc((size_t)d * sizeof(double));
    for (int64_t i = 0; i < d; ++i) mean[i] = sum[i] / (double)q.count;
    q.cost = node_cost(t, q.lower, mean) + node_cost(t, q.upper, mean);
    free(mean);
  }
  int64_t id = add_node(t);
  t->nodes[id] = q;
  memcpy(t->center + id * d, center, (size_t)d * sizeof(double));
  memcpy(t->radius + id * d, radius, (size_t)d * sizeof(double));
  memcpy(t->sum + id * d, sum, (size_t)d * sizeof(double));
  free(lb); free(ub); free(center); free(radius); free(sum);
  return id;
}

static void tree_new(tree *t, const mat *m) { /* BBDTree::new (bbd_tree.rs:42-60) */
  memset(t, 0, sizeof *t);
  t->d = m->d;
  t->index = malloc((size_t)m->n * sizeof(int64_t) + 1);
  for (int64_t i = 0; i < m->n; ++i) t->index[i] = i;
  t->root = m->n > 0 ? build_node(t, m, 0, m->n) : -1;
}

static void tree_free(tree *t) {
  free(t->nodes); free(t->center); free(t->radius); free(t->sum); free(t->index);
}

/* prune (bbd_tree.rs:165-193) */
static int prune(const double *center, const double *radius, const double *cents,
                 int64_t d, int64_t best, int64_t test) {
  if (best == test) return 0;
  const double *b = cents + best * d, *tt = cents + test * d;
  double lhs = 0.0, rhs = 0.0;
  for (int64_t i = 0; i < d; ++i) {
    double diff = tt[i] - b[i];
    lhs += diff * diff;
    if (diff > 0.0) rhs += (center[i] + radius[i] - b[i]) * diff;
    else rhs += (center[i] - radius[i] - b[i]) * diff;
  }
  return lhs >= 2.0 * rhs;
}

/* filter (bbd_tree.rs:89-163) */
static double filter(const tree *t, int64_t nd, const double *cents,
                     const int64_t *cand, int64_t k, double *sums,
                     int64_t *counts, int64_t *membership) {
  int64_t d = t->d;
  const double *center = t->center + nd * d;
  double min_dist = sqd_f64(center, cents + cand[0] * d, d);
  int64_t closest = cand[0];
  for (int64_t i = 1; i < k; ++i) {
    double dist = sqd_f64(center, cents + cand[i] * d, d);
    if (dist < min_dist) { min_dist = dist; closest = cand[i]; }
  }
  const node *q = &t->nodes[nd];
  if (q->lower >= 0) {
    int64_t *nc = malloc((size_t)k * sizeof(int64_t));
    int64_t newk = 0;
    for (int64_t i = 0; i < k; ++i)
      if (!prune(center, t->radius + nd * d, cents, d, closest, cand[i])) nc[newk++] = cand[i];
    if (newk > 1) {
      double a = filter(t, q->lower, cents, nc, newk, sums, counts, membership);
      double b = filter(t, q->upper, cents, nc, newk, sums, counts, membership);
      free(nc);
      return a + b;
    }
    free(nc);
  }
  const double *s = t->sum + nd * d;
  for (int64_t i = 0; i < d; ++i) sums[closest * d + i] += s[i];
  counts[closest] += q->count;
  for (int64_t i = q->index; i < q->index + q->count; ++i) membership[t->index[i]] = closest;
  return node_cost(t, nd, cents + closest * d);
}

/* clustering (bbd_tree.rs:62-87) */
static double clustering(const tree *t, const double *cents, int64_t k,
                         double *sums, int64_t *counts, int64_t *membership) {
  int64_t *cand = malloc((size_t)k * sizeof(int64_t));
  for (int64_t i = 0; i < k; ++i) { counts[i] = 0; cand[i] = i; }
  memset(sums, 0, (size_t)(k * t->d) * sizeof(double));
  double r = filter(t, t->root, cents, cand, k, sums, counts, membership);
  free(cand);
  return r;
}

double orc_bbd_clustering(int dtype, int layout, const void *x, int64_t n,
                          int64_t d, int64_t ld, const double *centroids,
                          int64_t k, double *sums, int64_t *counts,
                          int64_t *membership) {
  mat m = {dtype, layout, x, n, d, ld};
  tree t;
  tree_new(&t, &m);
  double r = clustering(&t, centroids, k, sums, counts, membership);
  tree_free(&t);
  return r;
}

/* ---- KMeans::fit (src/cluster/kmeans.rs:254-323) ---- */
int orc_kmeans_fit(int dtype, int layout, const void *x, int64_t n, int64_t d,
                   int64_t ld, int64_t k, int64_t max_iter, int64_t first_index,
                   const double *uniforms, double *centroids, int64_t *size,
                   int64_t *y, double *distortion_out, int64_t *iters,
                   double *dist_trace) {
  if (k < 2) {
    snprintf(g_err, sizeof g_err, "Fit failed: invalid number of clusters: %lld", (long long)k);
    return 1;
  }
  if (max_iter == 0) {
    snprintf(g_err, sizeof g_err, "Fit failed: invalid maximum number of iterations: %lld",
             (long long)max_iter);
    return 1;
  }
  mat m = {dtype, layout, x, n, d, ld};
  tree t;
  tree_new(&t, &m); /* built before validation in the reference; order is immaterial here */
  double distortion = DBL_MAX;
  orc_kmeanspp(dtype, layout, x, n, d, ld, k, first_index, uniforms, y, NULL);
  for (int64_t i = 0; i < k; ++i) size[i] = 0;
  memset(centroids, 0, (size_t)(k * d) * sizeof(double));
  for (int64_t i = 0; i < n; ++i) size[y[i]] += 1;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < d; ++j) centroids[y[i] * d + j] += getd(&m, i, j);
  for (int64_t i = 0; i < k; ++i)
    for (int64_t j = 0; j < d; ++j) centroids[i * d + j] /= (double)size[i];
  double *sums = calloc((size_t)(k * d), sizeof(double));
  int64_t it = 0;
  for (int64_t step = 1; step <= max_iter; ++step) {
    double dist = clustering(&t, centroids, k, sums, size, y);
    ++it;
    if (dist_trace) dist_trace[step - 1] = dist;
    for (int64_t i = 0; i < k; ++i)
      if (size[i] > 0)
        for (int64_t j = 0; j < d; ++j) centroids[i * d + j] = sums[i * d + j] / (double)size[i];
    if (distortion <= dist) break;
    distortion = dist;
  }
  *distortion_out = distortion;
  *iters = it;
  free(sums);
  tree_free(&t);
  return 0;
}

/* ---- KMeans::predict (src/cluster/kmeans.rs:327-352) ---- */
void orc_kmeans_predict(int dtype, int layout, const void *x, int64_t n,
                        int64_t d, int64_t ld, const double *centroids,
                        int64_t k, int64_t *labels) {
  mat m = {dtype, layout, x, n, d, ld};
  double *row = malloc((size_t)d * sizeof(double) + 8);
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t j = 0; j < d; ++j) row[j] = getd(&m, i, j);
    double min_dist = DBL_MAX;
    int64_t best = 0;
    for (int64_t c = 0; c < k; ++c) {
      double dist = sqd_f64(row, centroids + c * d, d);
      if (dist < min_dist) { min_dist = dist; best = c; }
    }
    labels[i] = best;
  }
  free(row);
}

/* Brute-force Lloyd loop: predict's assignment, sums in point order, the
 * distortion as the point-order sum of the winning distances, and fit's
 * break rule (kmeans.rs:305-309).  An independent label check only. */
void orc_lloyd_bruteforce(int dtype, int layout, const void *x, int64_t n,
                          int64_t d, int64_t ld, int64_t k, int64_t max_iter,
                          double *centroids, int64_t *size, int64_t *y,
                          double *distortion_out, int64_t *iters) {
  mat m = {dtype, layout, x, n, d, ld};
  double *row = malloc((size_t)d * sizeof(double) + 8);
  double *sums = malloc((size_t)(k * d) * sizeof(double) + 8);
  double distortion = DBL_MAX;
  int64_t it = 0;
  for (int64_t step = 1; step <= max_iter; ++step) {
    memset(sums, 0, (size_t)(k * d) * sizeof(double));
    for (int64_t c = 0; c < k; ++c) size[c] = 0;
    double dist = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      for (int64_t j = 0; j < d; ++j) row[j] = getd(&m, i, j);
      double md = DBL_MAX;
      int64_t best = 0;
      for (int64_t c = 0; c < k; ++c) {
        double v = sqd_f64(row, centroids + c * d, d);
        if (v < md) { md = v; best = c; }
      }
      y[i] = best;
      size[best] += 1;
      dist += md;
      for (int64_t j = 0; j < d; ++j) sums[best * d + j] += row[j];
    }
    ++it;
    for (int64_t c = 0; c < k; ++c)
      if (size[c] > 0)
        for (int64_t j = 0; j < d; ++j) centroids[c * d + j] = sums[c * d + j] / (double)size[c];
    if (distortion <= dist) break;
    distortion = dist;
  }
  *distortion_out = distortion;
  *iters = it;
  free(row); free(sums);
}

/* Timing harness for the CPU baseline: builds the BBD tree once, then runs
 * `iters` Lloyd iterations of KMeans::fit's loop body (kmeans.rs:295-303:
 * clustering + centroid update; the break rule is not applied) from the
 * given centroids, recording each iteration's wall time in iter_seconds. */
static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double orc_bbd_lloyd_timed(int dtype, int layout, const void *x, int64_t n,
                           int64_t d, int64_t ld, int64_t k, int64_t iters,
                           double *centroids, int64_t *labels,
                           double *iter_seconds) {
  mat m = {dtype, layout, x, n, d, ld};
  double t0 = now_s();
  tree t;
  tree_new(&t, &m);
  double build = now_s() - t0;
  double *sums = calloc((size_t)(k * d), sizeof(double));
  int64_t *size = calloc((size_t)k, sizeof(int64_t));
  for (int64_t it = 0; it < iters; ++it) {
    double a = now_s();
    clustering(&t, centroids, k, sums, size, labels);
    for (int64_t i = 0; i < k; ++i)
      if (size[i] > 0)
        for (int64_t j = 0; j < d; ++j) centroids[i * d + j] = sums[i * d + j] / (double)size[i];
    iter_seconds[it] = now_s() - a;
  }
  free(sums); free(size);
  tree_free(&t);
  return build;
}
