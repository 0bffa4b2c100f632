/*
 * smartcore_gb300 — C ABI of the GB300 (sm_103a) distance-argmin path of
 * smartcore 0.4.0: the Lloyd loop of KMeans::fit / KMeans::predict and the
 * brute-force LinearKNNSearch::find behind KNNClassifier / KNNRegressor.
 *
 * Conventions
 *   - Plain pointers and sizes only.  Sizes are int64_t (Rust usize);
 *     labels and neighbour indices are int64_t (usize), -1 for "None".
 *   - Matrices: element (i, j) of an n x d matrix is x[i*ld + j] for
 *     SC_ROW_MAJOR and x[j*ld + i] for SC_COL_MAJOR (DenseMatrix keeps both,
 *     column-major by default: src/linalg/basic/matrix.rs:187-238, :367-381).
 *   - Every call is blocking on the handle's own CUDA stream unless stated.
 *     Handles are not thread-safe; different handles may be used from
 *     different threads.
 *   - Errors: every entry point returns sc_status; sc_last_error() gives the
 *     message of the calling thread's last failure.  Parameter validation
 *     keeps the reference's messages (src/cluster/kmeans.rs:257-269,
 *     src/algorithm/neighbour/linear_search.rs:53-58) so a Rust shim can map
 *     SC_ERR_INVALID to Failed::fit / Failed::because(FindFailed, ...)
 *     (src/error/mod.rs:47-91) unchanged.
 *   - The GPU is required: there is no CPU fallback.  Without a usable
 *     CUDA device every compute call returns SC_ERR_CUDA.
 */
#ifndef SMARTCORE_GB300_H
#define SMARTCORE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t sc_status;
#define SC_OK 0
#define SC_ERR_INVALID 1  /* bad argument; message follows the reference */
#define SC_ERR_CUDA 2     /* CUDA runtime / launch failure, or no GPU */
#define SC_ERR_OOM 3      /* device allocation failed */
#define SC_ERR_TIMEOUT 4  /* a bounded device-side wait ran out */
#define SC_ERR_INTERNAL 5 /* a device-side consistency check failed */

#define SC_F32 0
#define SC_F64 1
#define SC_ROW_MAJOR 0
#define SC_COL_MAJOR 1
#define SC_MEM_HOST 0   /* pointer is host memory (pageable or pinned) */
#define SC_MEM_DEVICE 1 /* pointer is device memory of the current device */

/* Arithmetic form of the distance step.
 *   SC_FORM_FP64: every distance in FP64 with the reference's own operation
 *     order (src/metrics/distance/euclidian.rs:51-67).
 *   SC_FORM_SPLIT_BF16: -2 x.c^T as a split-BF16 tcgen05 GEMM (FP32
 *     accumulate) plus ||x||^2 + ||c||^2, with a certified error bound; every
 *     decision inside the bound is re-scored in FP64.  Results are identical
 *     to SC_FORM_FP64. */
#define SC_FORM_FP64 0
#define SC_FORM_SPLIT_BF16 1

/* Random generator behind get_rng_impl (src/rand_custom.rs:1-32). */
#define SC_RNG_SMALL 0 /* default features: rand 0.8 SmallRng (xoshiro256++) */
#define SC_RNG_STD 1   /* feature std_rand: rand 0.8 StdRng (ChaCha12) */

#define SC_KNN_UNIFORM 0  /* KNNWeightFunction::Uniform (src/neighbors/mod.rs:53-59) */
#define SC_KNN_DISTANCE 1 /* KNNWeightFunction::Distance */

/* Message of the calling thread's last failed call ("" if none). */
const char *sc_last_error(void);
/* ABI version of this library (major * 100 + minor). */
int32_t sc_abi_version(void);
/* 1 if a CUDA device of compute capability 10.3 is usable, else 0. */
int32_t sc_device_ok(void);
/* Number of CUDA kernels this library has launched in this process. */
int64_t sc_kernel_launches(void);

/* ------------------------------------------------------------------ */
/* k-means++ draws                                                     */
/* ------------------------------------------------------------------ */
/* The random draws of KMeans::kmeans_plus_plus (src/cluster/kmeans.rs:354-
 * 413) do not depend on the data: gen_range(0..n) once (:359), then
 * gen::<f64>() once per further seed (:385).  A Rust shim draws them with the
 * crate's own get_rng_impl(seed) and passes them in; this helper restates the
 * same rand 0.8.5 generators for non-Rust callers.  uniforms has k-1 slots. */
sc_status sc_kmeanspp_draws(int32_t rng, uint64_t seed, int64_t n, int64_t k,
                            int64_t *first_index, double *uniforms);

/* ------------------------------------------------------------------ */
/* KMeans                                                              */
/* ------------------------------------------------------------------ */
/* One-call KMeans::fit (src/cluster/kmeans.rs:254-323): k-means++ seeding
 * from the given draws, initial centroids = means of the seeding partition
 * (:275-292), then up to max_iter Lloyd iterations that stop when the
 * distortion did not strictly decrease (:305-309).  Replaces the BBDTree
 * filtering step (src/algorithm/neighbour/bbd_tree.rs:62-163) by a
 * brute-force assignment with the same labels.
 * x: n x d, host memory.  Outputs (host): centroids k*d (row-major),
 * sizes k, labels n, the final distortion and the number of iterations run.
 * SC_ERR_INVALID with "invalid number of clusters: {k}" for k < 2 and
 * "invalid maximum number of iterations: {max_iter}" for max_iter == 0. */
sc_status sc_kmeans_fit(const void *x, int32_t dtype, int32_t layout, int64_t n,
                        int64_t d, int64_t ld, int64_t k, int64_t max_iter,
                        int64_t first_index, const double *uniforms,
                        int32_t form, double *centroids_out, int64_t *sizes_out,
                        int64_t *labels_out, double *distortion_out,
                        int64_t *iters_out);

/* KMeans::predict (src/cluster/kmeans.rs:327-352): label of the nearest
 * centroid (strict <, lowest index wins ties) for each row of x (host). */
sc_status sc_kmeans_predict(const void *x, int32_t dtype, int32_t layout,
                            int64_t n, int64_t d, int64_t ld,
                            const double *centroids, int64_t k, int32_t form,
                            int64_t *labels_out);

/* Handle API: data resident on the device across calls. */
typedef struct sc_kmeans sc_kmeans;
/* Copies x (host or device memory, see mem) into a row-major device copy. */
sc_status sc_kmeans_create(const void *x, int32_t dtype, int32_t layout,
                           int32_t mem, int64_t n, int64_t d, int64_t ld,
                           int32_t form, sc_kmeans **out);
/* k-means++ on the device (kmeans.rs:354-413) plus the initial means. */
sc_status sc_kmeans_seed(sc_kmeans *h, int64_t k, int64_t first_index,
                         const double *uniforms);
/* Sets k and the current centroids (host, k*d row-major) directly. */
sc_status sc_kmeans_set_centroids(sc_kmeans *h, int64_t k,
                                  const double *centroids);
/* Runs Lloyd iterations.  stop_on_converge = 1: the reference loop (at most
 * max_iter iterations, break rule of kmeans.rs:305-309).  0: exactly
 * max_iter full iterations with the break rule disabled (throughput runs).
 * iters_done may be NULL; otherwise the call waits for completion.  With
 * more than two iterations the later ones replay the second captured as a
 * CUDA graph on the handle's stream (not when the caller is capturing that
 * stream, or with per-step timing on). */
sc_status sc_kmeans_iterate(sc_kmeans *h, int64_t max_iter,
                            int32_t stop_on_converge, int64_t *iters_done);
/* Copies the state to host buffers (any may be NULL). */
sc_status sc_kmeans_get(sc_kmeans *h, double *centroids, int64_t *sizes,
                        int64_t *labels, double *distortion, int64_t *iters);
/* The handle's CUDA stream (a cudaStream_t), for event timing. */
void *sc_kmeans_stream(sc_kmeans *h);
/* Counters of the last sc_kmeans_iterate: near-tie points re-scored in FP64
 * (split form) and k-means++ draws that needed the sequential replay. */
sc_status sc_kmeans_stats(sc_kmeans *h, int64_t *rescored, int64_t *pp_replays);
/* Steps of the last sc_kmeans_iterate whose cluster sums were updated from
 * the rows that changed label alone.  The sums are exact fixed-point
 * integers, so moving a row's values from its old cluster's sum to its new
 * one gives the same sums as summing every row again; a step takes that path
 * when at most 1/32 of the rows changed label (f32 data). */
sc_status sc_kmeans_sum_stats(sc_kmeans *h, int64_t *incremental_steps);
/* Timing of the assignment kernel: with profiling enabled, every Lloyd
 * iteration records a CUDA event pair on the handle's stream around its
 * assignment kernel; profile_read returns the summed elapsed time and the
 * number of timed launches since the last read (and resets them). */
sc_status sc_kmeans_profile(sc_kmeans *h, int32_t enable);
sc_status sc_kmeans_profile_read(sc_kmeans *h, double *total_ms,
                                 int64_t *launches);
sc_status sc_kmeans_sync(sc_kmeans *h);
void sc_kmeans_destroy(sc_kmeans *h);

/* One Lloyd iteration of the FP64 form that allocates nothing.  No
 * counterpart in the reference: it is the body of the loop in KMeans::fit
 * (src/cluster/kmeans.rs:294-310) as one call on buffers the caller owns.
 *
 * For callers that cannot allocate device memory during the call: a process
 * whose device memory is already reserved by its own pool allocator (a
 * cudaMalloc would fail or fragment that pool), or a loop that re-clusters
 * at a high rate, where cudaMalloc / cudaFree would take the CUDA driver's
 * allocation lock and cudaFree would synchronise the whole device.
 *
 * x          n x d row-major (ld = d) SC_F32 / SC_F64 matrix, device memory.
 * centroids  k x d row-major f64, device memory: read as the current
 *            centroids, overwritten with the new ones (an empty cluster
 *            keeps its centroid, kmeans.rs:297-303).
 * labels     n int32 labels out, device memory.
 * sizes      k int64 cluster sizes out, device memory, may be NULL.
 * distortion host pointer, may be NULL: sum over points of the FP64 squared
 *            distance to the assigned (old) centroid.
 * stream     cudaStream_t to run on (NULL: the legacy default stream).
 * Results are identical to sc_kmeans_set_centroids + one sc_kmeans_iterate
 * (max_iter 1, stop_on_converge 0) + sc_kmeans_get with SC_FORM_FP64.
 *
 * Scratch is a 1.6 MB static device array of this library, one per device,
 * so the limits are k <= 4096, k*d <= 65536 and n <= 8,388,608; larger
 * problems return SC_ERR_INVALID with the limit in the message.  The call
 * clears the parts of the scratch that must start at zero before it uses
 * them.  Every call in the process shares that array: overlapping calls on
 * one device would race on it, so calls are serialised by a process-wide
 * lock and each returns only after its work on the stream has finished.
 * The first call on each device (and CUDA context) looks the array's address
 * up with cudaGetSymbolAddress, which may load the library's device code.
 * Every call synchronises the stream twice (it reads max |x| back to pick
 * the fixed-point scale of the sums, and waits for its results), so it
 * cannot be used inside stream capture. */
sc_status sc_kmeans_step_noalloc(const void *x, int32_t dtype, int64_t n,
                                 int64_t d, double *centroids, int64_t k,
                                 int32_t *labels, int64_t *sizes,
                                 double *distortion, void *stream);

/* ------------------------------------------------------------------ */
/* Many independent KMeans::fit problems in one call                    */
/* ------------------------------------------------------------------ */
/* One problem of sc_kmeans_fit_batched: the arguments of sc_kmeans_fit
 * (inputs in host memory) plus its outputs and counters. */
typedef struct sc_kmeans_problem {
  const void *x;           /* n x d, host memory */
  int32_t layout;          /* SC_ROW_MAJOR or SC_COL_MAJOR */
  int32_t status;          /* out: SC_OK, or the error of this problem */
  int64_t n, d, ld;
  int64_t k, max_iter;
  int64_t first_index;     /* k-means++ draws, as for sc_kmeans_fit */
  const double *uniforms;  /* k - 1 entries */
  double *centroids_out;   /* k * d row-major, may be NULL */
  int64_t *sizes_out;      /* k, may be NULL */
  int64_t *labels_out;     /* n, may be NULL */
  double *distortion_out;  /* 1, may be NULL */
  int64_t *iters_out;      /* 1, may be NULL */
  int64_t rescored;        /* out: rows re-scored in FP64 */
  int64_t pp_replays;      /* out: k-means++ draws resolved by the replay */
} sc_kmeans_problem;

/* KMeans::fit (src/cluster/kmeans.rs:254-323) for `count` independent
 * problems of uneven n, d and k (all of element type dtype) in one call, each
 * with the results sc_kmeans_fit gives it alone (labels, sizes and iteration
 * count equal; centroids equal up to the rounding of the exact sums, within
 * 1e-15 relative).  Problems with d <= 64 and k <= 128 run together: every
 * problem's k-means++ draw j in one pair of launches, then a persistent
 * assignment kernel fed by a device work queue of (problem, rows) items and a
 * per-problem finalize, the Lloyd loop captured as a CUDA graph.  The others
 * run one after another through sc_kmeans_fit in `form`.
 * Every problem is validated first, with KMeans::fit's messages
 * (kmeans.rs:257-269) prefixed by "problem <i>: "; on a validation error
 * nothing runs and no output is written. */
sc_status sc_kmeans_fit_batched(sc_kmeans_problem *problems, int64_t count,
                                int32_t dtype, int32_t form);
/* Tuning of the batched assignment kernel: times its variants (centroids per
 * inner pass, rows per work item) on one synthetic problem per (d class,
 * k class), its items repeated so that every CTA has work, on the current
 * device and keeps the fastest for this process;
 * with path non-NULL also writes the table there.  Without a table the
 * batched call uses fixed defaults. */
sc_status sc_batch_tune(const char *path);
/* Loads a table written by sc_batch_tune; SC_ERR_INVALID when the file is
 * not one, is incomplete, or was made on another kind of device. */
sc_status sc_batch_tune_load(const char *path);
/* The variant the batched call uses for a problem of d features and k
 * clusters (centroids per inner pass, rows per work item). */
sc_status sc_batch_tune_get(int32_t d, int32_t k, int32_t *cu_out, int32_t *rows_out);

/* ------------------------------------------------------------------ */
/* Brute-force kNN (LinearKNNSearch)                                   */
/* ------------------------------------------------------------------ */
typedef struct sc_knn sc_knn;
/* LinearKNNSearch::new (src/algorithm/neighbour/linear_search.rs:45-47) over
 * the n training rows of train (host or device memory). */
sc_status sc_knn_create(const void *train, int32_t dtype, int32_t layout,
                        int32_t mem, int64_t n, int64_t d, int64_t ld,
                        sc_knn **out);
/* LinearKNNSearch::find (linear_search.rs:52-84) for m query rows at once.
 * Row q of idx_out / dist_out (m x k, host or device per out_mem) is the
 * reference's heap array in its own order: idx = training row, dist =
 * sqrt of the element-type squared distance; an empty slot is -1 / +inf.
 * SC_ERR_INVALID with "k should be >= 1 and <= length(data)" otherwise. */
sc_status sc_knn_find(sc_knn *h, const void *queries, int32_t layout,
                      int32_t mem, int64_t m, int64_t ld, int64_t k,
                      int32_t form, int32_t out_mem, int64_t *idx_out,
                      double *dist_out);
/* LinearKNNSearch::find_radius (linear_search.rs:89-108) for m query rows:
 * every training row i with d = sqrt(D) <= radius, in index order.
 * counts_out (host, m, may be NULL) receives each query's count and
 * total_out (may be NULL) their sum.  With idx_out / dist_out (host) non-NULL
 * and capacity >= total, they receive the rows of query 0, then of query 1,
 * ...; with both NULL only the counts are computed (call again with enough
 * capacity).  SC_ERR_INVALID with "radius should be > 0" (:90-95), or when
 * capacity < total (total_out is still set). */
sc_status sc_knn_find_radius(sc_knn *h, const void *queries, int32_t layout,
                             int32_t mem, int64_t m, int64_t ld, double radius,
                             int32_t form, int64_t *counts_out, int64_t capacity,
                             int64_t *idx_out, double *dist_out,
                             int64_t *total_out);
/* DBSCAN::fit (src/cluster/dbscan.rs:274-366) over the handle's training
 * rows with the linear search: every row's find_radius(eps) neighbourhood on
 * the device, then the reference's expansion loop on the host in its own visit
 * order.  labels_out (host, n): the cluster index of each row, or -1 for
 * noise; n_clusters_out (may be NULL): the number of clusters.
 * SC_ERR_INVALID with "Invalid minPts" (min_samples < 1) or "Invalid radius: "
 * (eps <= 0), the reference's messages. */
sc_status sc_dbscan_fit(sc_knn *h, double eps, int64_t min_samples, int32_t form,
                        int64_t *labels_out, int64_t *n_clusters_out);
/* DBSCAN::predict (dbscan.rs:370-398) for m query rows against the handle's
 * training rows labelled by sc_dbscan_fit: the cluster with the most
 * neighbours within eps (first maximum; noise counted last), as cluster + 1,
 * or 0 when noise wins.  out: host, m. */
sc_status sc_dbscan_predict(sc_knn *h, const void *queries, int32_t layout,
                            int32_t mem, int64_t m, int64_t ld, double eps,
                            int32_t form, const int64_t *train_labels,
                            int64_t n_clusters, int64_t *out);
/* FastPair::new / closest_pair (src/algorithm/neighbour/fastpair.rs:59-182)
 * over the handle's training rows: neighbour_out[i] / distance_out[i] (host,
 * n, may be NULL) are the entry `distances[i]` of the reference, the nearest
 * later row j > i by squared distance (first minimum, the running best kept in
 * the element type), and for row n - 1 itself and the element type's maximum;
 * closest_out (2) and closest_distance_out: closest_pair().
 * SC_ERR_INVALID with "min number of rows should be 3" below three rows. */
sc_status sc_fastpair(sc_knn *h, int64_t *neighbour_out, double *distance_out,
                      int64_t *closest_out, double *closest_distance_out);
/* KNNClassifier / KNNRegressor aggregation on the device over a find()
 * result already in idx/dist (device memory of this handle, m x k):
 * y_class = class index per training row (KNNClassifier::fit,
 * src/neighbors/knn_classifier.rs:229-235); classes_out = winning class
 * index per query (knn_classifier.rs:279-299). */
sc_status sc_knn_classify(sc_knn *h, const void *queries, int32_t layout,
                          int32_t mem, int64_t m, int64_t ld, int64_t k,
                          int32_t form, int32_t weight, const int64_t *y_class,
                          int64_t n_classes, int64_t *classes_out);
/* KNNRegressor::predict (src/neighbors/knn_regressor.rs:254-282), f64 y. */
sc_status sc_knn_regress(sc_knn *h, const void *queries, int32_t layout,
                         int32_t mem, int64_t m, int64_t ld, int64_t k,
                         int32_t form, int32_t weight, const double *y,
                         double *out);
void *sc_knn_stream(sc_knn *h);
/* Number of candidates re-scored in FP64 by the last split-form find. */
sc_status sc_knn_stats(sc_knn *h, int64_t *rescored);
void sc_knn_destroy(sc_knn *h);

/* ------------------------------------------------------------------ */
/* Testing hooks (no counterpart in the reference)                     */
/* ------------------------------------------------------------------ */
/* Bound (ns) of the pipeline waits of this handle's split-form assignment
 * kernel (0: the default 2 s).  Every wait of the kernel is bounded; when one
 * runs out the kernel stops, waits (with the default bound) for the copies
 * and tensor-core work it has issued, frees its tensor memory, and marks the
 * step void: the next sc_kmeans_iterate returns SC_ERR_TIMEOUT and the handle
 * runs no further iteration.  A tiny bound makes that path run on purpose. */
sc_status sc_kmeans_set_wait_limit(sc_kmeans *h, int64_t ns);
/* After `after` more successful device allocations of the library, every
 * allocation fails with SC_ERR_OOM until the hook is reset (after < 0). */
sc_status sc_debug_fail_alloc_after(int64_t after);
/* Device allocations of the library not yet freed (stream-ordered frees
 * count as freed when issued). */
int64_t sc_debug_live_allocations(void);
/* Candidate slots per query of the split-BF16 find (cap <= 0 restores the
 * default, 6 k (1 + ln(n / k)) + 64 rounded up to 32, at least 256); queries
 * with more candidates are served by the streaming kernel afterwards.  A small
 * cap exercises that path. */
sc_status sc_debug_knn_candidate_cap(int64_t cap);
/* Queries per pass of the split-BF16 find (rounded down to whole query tiles
 * of 128 or 256; q <= 0 restores the default, as many as keep the candidate
 * lists within 2 GB).  A small value exercises the passes over query chunks. */
sc_status sc_debug_knn_chunk_queries(int64_t q);
/* Every problem of the batched call uses this assignment variant (2, 4 or
 * 8 centroids per inner pass; a negative value restores the tuning table's
 * choice). */
sc_status sc_debug_batch_variant(int32_t variant);

#ifdef __cplusplus
}
#endif
#endif
