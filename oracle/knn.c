/*
 * Oracle restatement of smartcore's brute-force kNN path: HeapSelection,
 * LinearKNNSearch::find / find_radius, the classifier / regressor
 * aggregation, DBSCAN over find_radius, and FastPair's initial closest
 * pairs.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>

/* PartialOrd on f64: Less / Equal / Greater, or none when a NaN is involved. */
static int lt(double a, double b) { return a < b; }
static int ge_or_eq(double a, double b) { return a == b || a > b; }

typedef struct {
  double dist;
  int64_t idx; /* -1 = None */
} kp;

/* sift_down (src/algorithm/sort/heap_select.rs:71-86): node kk has children
 * 2*kk and 2*kk+1 of the 0-based array, so the root's first child is itself. */
static void sift_down_kp(kp *h, int64_t kk, int64_t n) {
  while (2 * kk <= n) {
    int64_t j = 2 * kk;
    if (j < n && lt(h[j].dist, h[j + 1].dist)) ++j;
    if (ge_or_eq(h[kk].dist, h[j].dist)) break;
    if (j == kk) break; /* only reachable with a NaN at the root, where the reference spins */
    kp t = h[kk]; h[kk] = h[j]; h[j] = t;
    kk = j;
  }
}

/* heapify (heap_select.rs:42-50) */
static void heapify_kp(kp *h, int64_t n) {
  if (n <= 1) return;
  for (int64_t i = n / 2 - 1; i >= 0; --i) sift_down_kp(h, i, n - 1);
}

static void sift_down_d(double *h, int64_t kk, int64_t n) {
  while (2 * kk <= n) {
    int64_t j = 2 * kk;
    if (j < n && lt(h[j], h[j + 1])) ++j;
    if (ge_or_eq(h[kk], h[j])) break;
    if (j == kk) break;
    double t = h[kk]; h[kk] = h[j]; h[j] = t;
    kk = j;
  }
}

/* HeapSelection::add (heap_select.rs:25-40) with sort (:88-91): a stable
 * sort into descending order once the heap first holds k elements. */
int64_t orc_heap_add_sequence(const double *values, int64_t count, int64_t k,
                              double *heap_out) {
  int64_t n = 0, len = 0;
  double *h = malloc((size_t)(k > 0 ? k : 1) * sizeof(double));
  for (int64_t e = 0; e < count; ++e) {
    double v = values[e];
    if (n < k) {
      h[len++] = v;
      ++n;
      if (n == k) { /* stable insertion sort, descending */
        for (int64_t i = 1; i < len; ++i) {
          double x = h[i];
          int64_t j = i - 1;
          while (j >= 0 && h[j] < x) { h[j + 1] = h[j]; --j; }
          h[j + 1] = x;
        }
      }
    } else {
      ++n;
      if (v < h[0]) { h[0] = v; sift_down_d(h, 0, k - 1); }
    }
  }
  for (int64_t i = 0; i < len; ++i) heap_out[i] = h[i];
  free(h);
  return n;
}

/* Distance::distance for Euclidian (src/metrics/distance/euclidian.rs:69-73):
 * sqrt of the element-type squared distance. */
static double dist_row(int dtype, const void *a, const void *b, int64_t d) {
  return sqrt(orc_sqdist(dtype, a, b, d));
}

static const void *row_at(int dtype, const void *base, int64_t i, int64_t d) {
  return dtype == ORC_F32 ? (const void *)((const float *)base + i * d)
                          : (const void *)((const double *)base + i * d);
}

/* LinearKNNSearch::find (src/algorithm/neighbour/linear_search.rs:52-84).
 * Rows are contiguous (the classifier copies rows into Vec<Vec<T>>,
 * src/neighbors/knn_classifier.rs:224-227). */
int orc_knn_find(int dtype, const void *train, int64_t n, int64_t d,
                 const void *queries, int64_t m, int64_t k, int64_t *idx,
                 double *dist) {
  if (k < 1 || k > n) return 1;
  kp *h = malloc((size_t)k * sizeof(kp));
  for (int64_t q = 0; q < m; ++q) {
    const void *from = row_at(dtype, queries, q, d);
    for (int64_t s = 0; s < k; ++s) { h[s].dist = INFINITY; h[s].idx = -1; }
    /* k adds of +inf end with a stable sort of equal keys: order unchanged */
    for (int64_t i = 0; i < n; ++i) {
      double dd = dist_row(dtype, from, row_at(dtype, train, i, d), d);
      if (dd < h[0].dist) {
        h[0].dist = dd;
        h[0].idx = i;
        heapify_kp(h, k);
      }
    }
    for (int64_t s = 0; s < k; ++s) { idx[q * k + s] = h[s].idx; dist[q * k + s] = h[s].dist; }
  }
  free(h);
  return 0;
}

/* LinearKNNSearch::find_radius (linear_search.rs:89-108) */
int64_t orc_knn_find_radius(int dtype, const void *train, int64_t n, int64_t d,
                            const void *queries, int64_t m, double radius,
                            int64_t *counts, int64_t *idx, double *dist,
                            int64_t cap) {
  if (!(radius > 0.0)) return -1;
  int64_t total = 0;
  for (int64_t q = 0; q < m; ++q) {
    const void *from = row_at(dtype, queries, q, d);
    int64_t c = 0;
    for (int64_t i = 0; i < n; ++i) {
      double dd = dist_row(dtype, from, row_at(dtype, train, i, d), d);
      if (dd <= radius) {
        if (total >= cap) return -2;
        idx[total] = i;
        dist[total] = dd;
        ++total;
        ++c;
      }
    }
    counts[q] = c;
  }
  return total;
}

/* KNNWeightFunction::calc_weights (src/neighbors/mod.rs:62-78) over the
 * entries whose index is Some (find's flat_map, linear_search.rs:79-83). */
static int64_t weights(const int64_t *idx, const double *dist, int64_t k,
                       int weight, double *w, int64_t *pos) {
  int64_t c = 0;
  for (int64_t s = 0; s < k; ++s)
    if (idx[s] >= 0) pos[c++] = s;
  int any_zero = 0;
  for (int64_t t = 0; t < c; ++t) any_zero |= dist[pos[t]] == 0.0;
  for (int64_t t = 0; t < c; ++t) {
    double e = dist[pos[t]];
    if (weight == 0) w[t] = 1.0;
    else if (any_zero) w[t] = e == 0.0 ? 1.0 : 0.0;
    else w[t] = 1.0 / e;
  }
  return c;
}

/* KNNClassifier::predict_for_row (src/neighbors/knn_classifier.rs:279-299) */
void orc_knn_vote(const int64_t *idx, const double *dist, int64_t m, int64_t k,
                  const int64_t *y, int64_t n_classes, int weight,
                  int64_t *class_out) {
  double *w = malloc((size_t)k * sizeof(double));
  int64_t *pos = malloc((size_t)k * sizeof(int64_t));
  double *c = malloc((size_t)(n_classes > 0 ? n_classes : 1) * sizeof(double));
  for (int64_t q = 0; q < m; ++q) {
    const int64_t *qi = idx + q * k;
    int64_t cnt = weights(qi, dist + q * k, k, weight, w, pos);
    double w_sum = 0.0;
    for (int64_t t = 0; t < cnt; ++t) w_sum += w[t];
    for (int64_t j = 0; j < n_classes; ++j) c[j] = 0.0;
    double max_c = 0.0;
    int64_t max_i = 0;
    for (int64_t t = 0; t < cnt; ++t) {
      int64_t cls = y[qi[pos[t]]];
      c[cls] += w[t] / w_sum;
      if (c[cls] > max_c) { max_c = c[cls]; max_i = cls; }
    }
    class_out[q] = max_i;
  }
  free(w); free(pos); free(c);
}

/* KNNRegressor::predict_for_row (src/neighbors/knn_regressor.rs:268-282), TY = f64 */
void orc_knn_regress(const int64_t *idx, const double *dist, int64_t m,
                     int64_t k, const double *y, int weight, double *out) {
  double *w = malloc((size_t)k * sizeof(double));
  int64_t *pos = malloc((size_t)k * sizeof(int64_t));
  for (int64_t q = 0; q < m; ++q) {
    const int64_t *qi = idx + q * k;
    int64_t cnt = weights(qi, dist + q * k, k, weight, w, pos);
    double w_sum = 0.0;
    for (int64_t t = 0; t < cnt; ++t) w_sum += w[t];
    double r = 0.0;
    for (int64_t t = 0; t < cnt; ++t) r += y[qi[pos[t]]] * (w[t] / w_sum);
    out[q] = r;
  }
  free(w); free(pos);
}

/* find_radius of row `from` as a growing index list (linear_search.rs:89-108) */
static int64_t radius_list(int dtype, const void *x, int64_t n, int64_t d, const void *from, double eps,
                           int64_t **buf, int64_t *cap) {
  int64_t c = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (dist_row(dtype, from, row_at(dtype, x, i, d), d) <= eps) {
      if (c == *cap) {
        *cap = *cap ? 2 * *cap : 64;
        *buf = realloc(*buf, (size_t)*cap * sizeof(int64_t));
      }
      (*buf)[c++] = i;
    }
  }
  return c;
}

/* DBSCAN::fit (src/cluster/dbscan.rs:274-366) with LinearKNNSearch: y[i] is
 * the cluster of row i or -1 (outlier).  Returns the number of clusters, -1
 * for min_samples < 1 ("Invalid minPts"), -2 for eps <= 0 ("Invalid radius").
 * find_radius is called exactly where the reference calls it. */
int64_t orc_dbscan_fit(int dtype, const void *x, int64_t n, int64_t d, double eps, int64_t min_samples,
                       int64_t *y) {
  if (min_samples < 1) return -1;
  if (!(eps > 0.0)) return -2;
  const int64_t queued = -2, outlier = -1, undefined = -3;
  for (int64_t i = 0; i < n; ++i) y[i] = undefined;
  int64_t *nb = NULL, *sec = NULL, nb_cap = 0, sec_cap = 0;
  int64_t k = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (y[i] != undefined) continue;
    int64_t len = radius_list(dtype, x, n, d, row_at(dtype, x, i, d), eps, &nb, &nb_cap);
    if (len < min_samples) {
      y[i] = outlier;
      continue;
    }
    y[i] = k;
    for (int64_t j = 0; j < len; ++j)
      if (y[nb[j]] == undefined) y[nb[j]] = queued;
    while (len > 0) { /* neighbors.pop(): last element first */
      const int64_t index = nb[--len];
      if (y[index] == outlier) y[index] = k;
      if (y[index] == undefined || y[index] == queued) {
        y[index] = k;
        const int64_t ns = radius_list(dtype, x, n, d, row_at(dtype, x, index, d), eps, &sec, &sec_cap);
        if (ns >= min_samples) {
          for (int64_t j = 0; j < ns; ++j) {
            const int64_t label = y[sec[j]];
            if (label == undefined) y[sec[j]] = queued;
            if (label == undefined || label == outlier) {
              if (len == nb_cap) {
                nb_cap = nb_cap ? 2 * nb_cap : 64;
                nb = realloc(nb, (size_t)nb_cap * sizeof(int64_t));
              }
              nb[len++] = sec[j];
            }
          }
        }
      }
    }
    ++k;
  }
  free(nb);
  free(sec);
  return k;
}

/* DBSCAN::predict (dbscan.rs:370-398): per query, votes over the training
 * rows within eps (noise last); which_max keeps the first maximum
 * (src/tree/decision_tree_classifier.rs:490-502); class + 1, or 0 for noise. */
void orc_dbscan_predict(int dtype, const void *x, int64_t n, int64_t d, const int64_t *y, int64_t k,
                        const void *q, int64_t m, double eps, int64_t *out) {
  int64_t *votes = malloc((size_t)(k + 1) * sizeof(int64_t));
  for (int64_t r = 0; r < m; ++r) {
    const void *from = row_at(dtype, q, r, d);
    for (int64_t c = 0; c <= k; ++c) votes[c] = 0;
    for (int64_t i = 0; i < n; ++i)
      if (dist_row(dtype, from, row_at(dtype, x, i, d), d) <= eps) ++votes[y[i] < 0 ? k : y[i]];
    int64_t which = 0;
    for (int64_t c = 1; c <= k; ++c)
      if (votes[c] > votes[which]) which = c;
    out[r] = which != k ? which + 1 : 0;
  }
  free(votes);
}

/* FastPair::init (src/algorithm/neighbour/fastpair.rs:82-150) step by step:
 * the map `distances` as arrays nb / dist (nb = -1 for None), `insert` and
 * `and_modify` as overwrites, the running best nbd kept in the element type
 * (T::from(d)).  Row n - 1 ends with neighbour n - 1 and T::MAX. */
int orc_fastpair(int dtype, const void *x, int64_t n, int64_t d, int64_t *nb, double *dist) {
  if (n < 3) return -1; /* "min number of rows should be 3" */
  const double tmax = dtype == ORC_F32 ? (double)FLT_MAX : DBL_MAX;
  for (int64_t i = 0; i < n - 1; ++i) { nb[i] = -1; dist[i] = tmax; }
  for (int64_t i = 0; i < n; ++i) {
    int64_t index_closest = i + 1;
    double nbd = dist[i];
    for (int64_t j = i + 1; j < n; ++j) {
      nb[j] = i;
      dist[j] = nbd;
      const double dd = orc_sqdist(dtype, row_at(dtype, x, i, d), row_at(dtype, x, j, d), d);
      if (dd < nbd) {
        index_closest = j;
        nbd = dtype == ORC_F32 ? (double)(float)dd : dd;
      }
    }
    dist[i] = nbd;
    nb[i] = index_closest;
  }
  nb[n - 1] = n - 1;
  dist[n - 1] = tmax;
  return 0;
}
