// Shared declarations of the smartcore_gb300 CUDA library.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/smartcore_gb300.h"

namespace sc {

// ---- host-side error reporting (thread-local message, see sc_last_error) ----
void set_error(const char *fmt, ...);
sc_status cuda_fail(cudaError_t e, const char *what);

#define SC_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return ::sc::cuda_fail(e_, #call);                \
  } while (0)

// Every kernel launch of the library is followed by SC_LAUNCHED(): it counts
// the launch (sc_kernel_launches) and surfaces launch errors.
void note_launch();
#define SC_LAUNCHED()                                                        \
  do {                                                                       \
    ::sc::note_launch();                                                     \
    SC_CUDA(cudaGetLastError());                                             \
  } while (0)

#define SC_TRY(expr)                                                         \
  do {                                                                       \
    sc_status s_ = (expr);                                                   \
    if (s_ != SC_OK) return s_;                                              \
  } while (0)

// Programmatic dependent launch.  A kernel launched by launch_pdl may start
// while the stream's previous kernel runs; it calls pdl_wait_prerequisite()
// before its first read of that kernel's results (and before any early
// exit), and pdl_release_dependents() to let its own successor come up.
// Launched the ordinary way, both are no-ops.
__device__ __forceinline__ void pdl_wait_prerequisite() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }
template <typename... KArgs, typename... Args>
sc_status launch_pdl(void (*kern)(KArgs...), int64_t grid, int threads, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  SC_CUDA(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
  return SC_OK;
}

// ---- device-resident state of one Lloyd loop ----
struct LloydState {
  double distortion;   // the reference's `distortion` (starts at f64::MAX)
  double last_dist;    // distortion of the most recent clustering step
  int64_t iters;       // clustering steps executed
  int64_t rescored;    // split form: points re-scored in FP64
  int64_t pp_replays;  // k-means++ draws resolved by the sequential replay
  int32_t done;        // break rule taken (kmeans.rs:305-309)
  int32_t stop;        // 1: apply the break rule; 0: run every iteration
  int32_t err;         // device-side consistency failure code (0 = none)
  int32_t sums_valid;  // the persistent cluster sums hold the sums of the previous labels
  int64_t pp_chosen;   // k-means++: row index of the current seed
  int64_t moved;       // rows whose label changed in the current step
  int64_t incremental_steps;  // steps whose sums were updated from the moved rows alone
};

// 128-bit fixed-point accumulator word pair (lo, hi), two's complement.
struct Acc128 {
  unsigned long long lo, hi;
};

constexpr int kMaxKnnK = 64;  // largest k served by the kNN kernels

// Buffers of the centroid-sum step.  mode 0: one 128-bit fixed-point
// accumulator per (cluster, feature) updated with global atomics.  mode 1:
// each CTA sorts its contiguous chunk of points by label and sums each
// cluster's rows as int64 fixed point, one partial per CTA (equal row slices
// per warp with shared-memory accumulators when k x d of them fit, else one
// warp per cluster); the finalize step adds the partials exactly in 128 bits.
// All are order independent, so every variant gives the same bits.
struct UpdateBuf {
  int mode = 0;
  int grid = 0;      // mode 1: number of CTAs (partials)
  int threads = 0;   // mode 1: threads per CTA
  int scale = 0;     // fixed-point scale 2^scale of the active mode
  size_t smem = 0;   // mode 1: dynamic shared memory per CTA
  size_t balanced_smem = 0;  // mode 1: shared memory of the balanced kernel (0: per-cluster warps)
  Acc128 *acc = nullptr;            // mode 0: k x d
  unsigned long long *cnt = nullptr;  // mode 0: k
  long long *part = nullptr;        // mode 1: grid x k x d
  unsigned int *cpart = nullptr;    // mode 1: grid x k
  uint32_t *xq = nullptr;           // mode 1: the points in the packed fixed-point form of `scale`
  const void *xq_src = nullptr;     // the points xq was made from
  bool xq_slow = false;             // some value of xq needs the conversion from f32
  // mode 1, incremental sums: the exact totals of the last step's labels
  // persist, and a step in which few labels change moves only those rows'
  // values between clusters (integer sums: the same totals as a full pass)
  Acc128 *tot = nullptr;            // k x d
  unsigned long long *tcnt = nullptr;  // k
  int32_t *prev = nullptr;          // n: the labels the totals were summed for
  int64_t *mrows = nullptr;         // moved rows of the step (at most mcap)
  int32_t *mold = nullptr;          //   and their previous labels
  int64_t mcap = 0;                 // moved rows above which the step runs the full pass
};

// ---- device memory ----
// Stream-ordered allocations from the device's default memory pool.  Its
// release threshold is raised once per device, so blocks a destroyed handle
// gave back serve the next handle without new driver mappings.  A block is
// freed in the order of the stream that last used it.
sc_status dev_alloc(void **p, size_t bytes, cudaStream_t s);
void dev_free(void *p, cudaStream_t s);
template <class T>
sc_status dalloc(T **p, size_t count, cudaStream_t s) {
  return dev_alloc((void **)p, (count ? count : 1) * sizeof(T), s);
}
template <class T>
void dfree(T *&p, cudaStream_t s) {
  dev_free((void *)p, s);
  p = nullptr;
}

// ---- kernel launchers (defined in the .cu files) ----
// exact.cu: FP64 forms with the reference's operation order.
sc_status launch_assign_fp64(int dtype, const void *x, int64_t n, int d,
                             const double *cent, int k, int32_t *labels,
                             double *part, const LloydState *st,
                             cudaStream_t s);
// seed_cc (k entries, may be null): lower bounds of the squared distances
// from the current seed to the earlier ones, written by launch_pp_select;
// dd32 (n entries, may be null): d rounded up to f32, the far test's copy
// (f32 rows with d <= 128 only); xh (may be null): the BF16 high halves of
// the rows (n_pad x d_pad, split form) with xnrm >= |x| per row.
sc_status launch_pp_update(int dtype, const void *x, int64_t n, int d,
                           const LloydState *st, int32_t label_of_seed,
                           double *dd, float *dd32, int32_t *labels, double *part,
                           int first_pass, const float *seed_cc, const __nv_bfloat16 *xh, int d_pad,
                           const float *xnrm, cudaStream_t s);
// Picks seed j into st->pp_chosen and its row into seed_x[j] (k x d, element
// type); writes seed_cc[0..j).
sc_status launch_pp_select(int dtype, const void *x, int d, const double *dd, const double *part,
                           int64_t n, int nb, const double *uniform, LloydState *st,
                           void *seed_x, float *seed_cc, int j, cudaStream_t s);
sc_status launch_knn_fp64(int dtype, const void *train, int64_t n, int d,
                          const void *queries, int64_t m, int k, int64_t *idx,
                          double *dist, cudaStream_t s);
sc_status launch_knn_radius_fp64(int dtype, const void *train, int64_t n, int d, const void *queries, int64_t m,
                                 double radius, int64_t *counts, const int64_t *offsets, int64_t *idx,
                                 double *dist, cudaStream_t s);
sc_status launch_widen_labels(const int32_t *in, int64_t *out, int64_t n, cudaStream_t s);
sc_status launch_fastpair(int dtype, const void *x, int64_t n, int d, int64_t *nb, double *dist,
                          cudaStream_t s);
sc_status launch_knn_vote(const int64_t *idx, const double *dist, int64_t m,
                          int k, int weight, const int64_t *y_class,
                          int64_t *out, cudaStream_t s);
sc_status launch_knn_regress(const int64_t *idx, const double *dist,
                             int64_t m, int k, int weight, const double *y,
                             double *out, cudaStream_t s);
int pp_block_count(int64_t n);
int assign_block_count(int64_t n);

// update.cu: centroid sums, counts and the end-of-iteration step.
sc_status launch_update_fixed(int dtype, const void *x, int64_t n, int d,
                              const int32_t *labels, Acc128 *acc,
                              unsigned long long *cnt, int scale,
                              const LloydState *st, cudaStream_t s);
sc_status launch_finalize_centroids(Acc128 *acc, unsigned long long *cnt,
                                    double *cent, int64_t *sizes, int k, int d,
                                    int scale, double *cluster_terms,
                                    int empty_nan, const LloydState *st,
                                    cudaStream_t s);
sc_status launch_finalize_scalar(const double *part, int nparts,
                                 const double *cluster_terms, int64_t nterms,
                                 const double *xnorm_total, LloydState *st,
                                 cudaStream_t s);
// Mode, fixed-point scale and partial count that update_alloc picks for
// (n, d, k); absmax = max |x|.  Every path that sums at the returned scale
// rounds each value to the same fixed-point integer, so equal inputs give
// equal centroids whichever buffers hold the sums.
struct UpdatePlan {
  int mode = 0, grid = 0, scale = 0;
  size_t smem = 0;
};
UpdatePlan update_plan(int dtype, int64_t n, int d, int k, double absmax, int num_sms);
// Chooses the mode for (n, d, k) and allocates; absmax = max |x|.
sc_status update_alloc(UpdateBuf *u, int dtype, int64_t n, int d, int k, double absmax, int num_sms,
                       cudaStream_t s);
// Number of distortion terms launch_finalize writes: one per cluster (mode 0)
// or one per block of 32 (cluster, feature) elements (mode 1).
inline int64_t update_nterms(const UpdateBuf *u, int k, int d) {
  return u->mode != 0 ? ((int64_t)k * d + 31) / 32 : k;
}
void update_free(UpdateBuf *u, cudaStream_t s);
// After a full pass outside the Lloyd loop (the seeding's initial means):
// the labels the totals now hold and the flag that makes the next step's
// incremental path available.
sc_status update_mark_sums(const UpdateBuf *u, const int32_t *labels, int64_t n, LloydState *st, cudaStream_t s);
// Packs the points for the balanced partial form (once per dataset and scale).
sc_status update_pack(UpdateBuf *u, const float *x, int64_t n, int d, cudaStream_t s);
sc_status launch_update(const UpdateBuf *u, int dtype, const void *x, int64_t n, int d,
                        const int32_t *labels, int k, const LloydState *st, cudaStream_t s);
sc_status launch_finalize(const UpdateBuf *u, double *cent, int64_t *sizes, int k, int d,
                          double *cluster_terms, int empty_nan, const LloydState *st,
                          cudaStream_t s);
sc_status launch_absmax(int dtype, const void *x, int64_t count,
                        unsigned long long *out_bits, cudaStream_t s);
sc_status launch_to_row_major(int dtype, const void *src, int64_t n, int64_t d,
                              int64_t ld, void *dst, cudaStream_t s);

}  // namespace sc
