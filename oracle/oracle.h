/*
 * CPU oracle for the distance-argmin path of smartcore 0.4.0.
 *
 * TEST INFRASTRUCTURE ONLY.  This library checks the product: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product library (libsmartcore_gb300.so) never links or calls it.
 *
 * Every function restates the reference algorithm in plain C11, compiled with
 * -ffp-contract=off so that no multiply-add is fused (rustc never fuses), and
 * cites the reference file:line it follows (paths relative to the smartcore
 * source tree).  Row-major or column-major inputs are accepted; element
 * (i, j) of an n x d matrix lives at x[i*ld + j] (row-major) or
 * x[j*ld + i] (column-major), mirroring DenseMatrix::get
 * (src/linalg/basic/matrix.rs:367-381).
 *
 * Parity pins: the reference's own known-answer tests (tests/golden/).  The
 * rand 0.8.5 restatement (SmallRng = xoshiro256++, StdRng = ChaCha12) is
 * "parity unpinned": no reference test fixes a seeded draw and the crate
 * cannot be built here.
 */
#ifndef SMARTCORE_ORACLE_H
#define SMARTCORE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_F32 = 0, ORC_F64 = 1 };
enum { ORC_ROW_MAJOR = 0, ORC_COL_MAJOR = 1 };
enum { ORC_RNG_SMALL = 0, ORC_RNG_STD = 1 };

/* ---- rand 0.8.5 (src/rand_custom.rs:8-32) ---- */
/* Draws of KMeans::kmeans_plus_plus (src/cluster/kmeans.rs:359, :385): one
 * gen_range(0..n) then k-1 gen::<f64>().  No reference test pins these. */
void orc_kmeanspp_draws(int rng_kind, uint64_t seed, int64_t n, int64_t k,
                        int64_t *first_index, double *uniforms /* k-1 */);
/* Raw next_u64 stream, for cross-checking two independent restatements. */
void orc_rng_u64(int rng_kind, uint64_t seed, int64_t count, uint64_t *out);
/* The primitives under the draws, exposed to be checked one by one against
 * the published algorithms' own known answers. */
void orc_xoshiro256pp(const uint64_t state[4], int64_t count, uint64_t *out);
void orc_splitmix64(uint64_t seed, int64_t count, uint64_t *out);
void orc_chacha_block(const uint32_t key[8], const uint32_t w12_15[4], int rounds, uint32_t out[16]);
void orc_chacha_quarter_round(uint32_t v[4]);
void orc_pcg32(uint64_t state, uint64_t inc, int after_step, int64_t count, uint32_t *out);

/* ---- Euclidian::squared_distance (src/metrics/distance/euclidian.rs:51-67) ---- */
double orc_sqdist(int dtype, const void *a, const void *b, int64_t d);

/* ---- KMeans (src/cluster/kmeans.rs) ---- */
/* Full KMeans::fit (kmeans.rs:254-323) with the BBD-tree filtering step
 * (src/algorithm/neighbour/bbd_tree.rs).  Returns 0, or 1 for invalid
 * parameters (k < 2, max_iter == 0; message via orc_last_error). */
int orc_kmeans_fit(int dtype, int layout, const void *x, int64_t n, int64_t d,
                   int64_t ld, int64_t k, int64_t max_iter, int64_t first_index,
                   const double *uniforms, double *centroids /* k*d */,
                   int64_t *sizes /* k */, int64_t *labels /* n */,
                   double *distortion, int64_t *iters,
                   double *dist_trace /* max_iter, may be NULL */);
/* KMeans::kmeans_plus_plus (kmeans.rs:354-413): labels of the nearest seed. */
void orc_kmeanspp(int dtype, int layout, const void *x, int64_t n, int64_t d,
                  int64_t ld, int64_t k, int64_t first_index,
                  const double *uniforms, int64_t *labels, int64_t *chosen /* k */);
/* KMeans::predict (kmeans.rs:327-352). */
void orc_kmeans_predict(int dtype, int layout, const void *x, int64_t n,
                        int64_t d, int64_t ld, const double *centroids,
                        int64_t k, int64_t *labels);
/* One BBDTree::clustering call (bbd_tree.rs:62-87) on a fresh tree. */
double orc_bbd_clustering(int dtype, int layout, const void *x, int64_t n,
                          int64_t d, int64_t ld, const double *centroids,
                          int64_t k, double *sums /* k*d */,
                          int64_t *counts, int64_t *membership);
/* Brute-force Lloyd loop with the same break rule, for independent label
 * checks at sizes where the tree is too large: assignment = KMeans::predict
 * arithmetic, sums in point order. */
void orc_lloyd_bruteforce(int dtype, int layout, const void *x, int64_t n,
                          int64_t d, int64_t ld, int64_t k, int64_t max_iter,
                          double *centroids /* in: initial, out: final */,
                          int64_t *sizes, int64_t *labels, double *distortion,
                          int64_t *iters);

/* CPU-baseline harness: BBD tree built once (returns its build seconds),
 * then `iters` untested Lloyd iterations from `centroids`, each timed. */
double orc_bbd_lloyd_timed(int dtype, int layout, const void *x, int64_t n,
                           int64_t d, int64_t ld, int64_t k, int64_t iters,
                           double *centroids, int64_t *labels,
                           double *iter_seconds);

/* ---- HeapSelection (src/algorithm/sort/heap_select.rs) ---- */
/* Feeds values through HeapSelection::add; writes the k-slot heap array
 * (heap.get()) and returns the element count n. */
int64_t orc_heap_add_sequence(const double *values, int64_t count, int64_t k,
                              double *heap_out);

/* ---- LinearKNNSearch (src/algorithm/neighbour/linear_search.rs) ---- */
/* find (linear_search.rs:52-84) for m queries.  Output row q holds the heap
 * array in heap order; an empty slot (index None) is -1 / +inf.
 * Returns 0, or 1 when k < 1 or k > n. */
int orc_knn_find(int dtype, const void *train, int64_t n, int64_t d,
                 const void *queries, int64_t m, int64_t k, int64_t *idx,
                 double *dist);
/* find_radius (linear_search.rs:89-108): counts[q] neighbours of query q,
 * appended to idx/dist in query order; returns total, or -1 if radius <= 0,
 * or -2 if cap is too small. */
int64_t orc_knn_find_radius(int dtype, const void *train, int64_t n, int64_t d,
                            const void *queries, int64_t m, double radius,
                            int64_t *counts, int64_t *idx, double *dist,
                            int64_t cap);
/* KNNClassifier::predict_for_row (src/neighbors/knn_classifier.rs:279-299)
 * over find() output.  y = class index per train row (fit, :229-235);
 * weight 0 = Uniform, 1 = Distance (src/neighbors/mod.rs:62-78). */
int64_t orc_dbscan_fit(int dtype, const void *x, int64_t n, int64_t d, double eps, int64_t min_samples,
                       int64_t *y);
void orc_dbscan_predict(int dtype, const void *x, int64_t n, int64_t d, const int64_t *y, int64_t k,
                        const void *q, int64_t m, double eps, int64_t *out);
int orc_fastpair(int dtype, const void *x, int64_t n, int64_t d, int64_t *nb, double *dist);
void orc_knn_vote(const int64_t *idx, const double *dist, int64_t m, int64_t k,
                  const int64_t *y, int64_t n_classes, int weight,
                  int64_t *class_out);
/* KNNRegressor::predict_for_row (src/neighbors/knn_regressor.rs:268-282). */
void orc_knn_regress(const int64_t *idx, const double *dist, int64_t m,
                     int64_t k, const double *y, int weight, double *out);

const char *orc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
